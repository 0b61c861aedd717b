#!/usr/bin/env python3
"""Regenerate the golden fixtures in tests/golden from the reference checkout.

Run in a container that has the reference at REFERENCE_ROOT (default
/root/reference); the GPU machine never runs this script, it only reads the
committed outputs:

  archive_digests.json   digests of the reference's archived task lists
                         (13Bit_codon/Archive/bin/constellations_N{6..21}_5.bin)
                         and per-constellation solutions
                         (solutions_N{6..19}_5_v2.bin), with counts and sums
  archive_small.npz      the archived solution records themselves for N=6..12
  ref_py_vectors.npz     per-record vectors from the reference's own Python host
                         functions (14Bit_codon_GPU/356Py_savesp_narrow.py:
                         gen_constellations, build_soa_for_range, dfs_iter)
                         executed under CPython, with a node counter added to
                         dfs_iter, for N=6..11 at presets 4..7 where valid
                         and for N=12 at presets 4 and 5
  ref_c_totals.json      totals printed by the reference's C restatement
                         (10Bit_CUDA/13CUDA_constellation.c, preset 4) built by
                         oracle/Makefile into oracle/_ref/ref13c
  ref_unique.json        (total, unique) of 11Bit_Python/07Py_bit_symmetry.py
                         executed under CPython for N=4..11

The reference's Python source is read and executed in memory (two Codon
`@par` lines become `pass`, u32/u64/u8 become masking functions); nothing of
it is written into this repository.
"""
from __future__ import annotations

import __future__
import ast
import importlib.util
import json
import os
import subprocess
import sys
import typing

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from golden_util import solution_digest, task_digest  # noqa: E402

REF = os.environ.get("REFERENCE_ROOT", "/root/reference")
ARCHIVE = os.path.join(REF, "13Bit_codon", "Archive", "bin")
PY356 = os.path.join(REF, "14Bit_codon_GPU", "356Py_savesp_narrow.py")
PY07 = os.path.join(REF, "11Bit_Python", "07Py_bit_symmetry.py")

HOST_FUNCS = ["to_ijkl", "mirvert", "ffmin", "geti", "getj", "getk", "getl", "rot90", "symmetry",
              "symmetry90", "check_rotations", "get_jasmin", "jasmin", "set_pre_queens_cached",
              "set_pre_queens", "gen_constellations", "build_soa_for_range", "dfs_iter",
              "select_dynamic_preset_queens", "_bit_total"]
HOST_GLOBALS = ["use_visited_prune", "DISABLE_CONSTELLATION_SIGNATURE_PRUNE", "jasmin_cache_global"]


class _NodeCounter(ast.NodeTransformer):
    """Adds `_NODES[0] += 1` after every `bit = avail & -avail` inside dfs_iter."""

    def visit_AnnAssign(self, node):
        if isinstance(node.target, ast.Name) and node.target.id == "bit":
            inc = ast.parse("_NODES[0] += 1").body[0]
            return [node, inc]
        return node


def load_reference_host():
    src = open(PY356).read().split("\n")
    src = [ln.replace("@par", "pass") if ln.strip() == "@par" else ln for ln in src]
    tree = ast.parse("\n".join(src))
    keep = []
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name in HOST_FUNCS:
            if node.name == "dfs_iter":
                node = _NodeCounter().visit(node)
            keep.append(node)
        elif isinstance(node, ast.ClassDef) and node.name == "TaskSoA":
            keep.append(node)
        elif isinstance(node, (ast.AnnAssign, ast.Assign)):
            tgt = node.target if isinstance(node, ast.AnnAssign) else node.targets[0]
            if isinstance(tgt, ast.Name) and tgt.id in HOST_GLOBALS:
                keep.append(node)
    mod = ast.Module(body=keep, type_ignores=[])
    ast.fix_missing_locations(mod)
    ns = {
        "u32": lambda x: int(x) & 0xFFFFFFFF,
        "u64": lambda x: int(x) & 0xFFFFFFFFFFFFFFFF,
        "u8": lambda x: int(x) & 0xFF,
        "List": typing.List, "Dict": typing.Dict, "Set": typing.Set, "Tuple": typing.Tuple,
        "_NODES": [0],
    }
    code = compile(mod, PY356, "exec", flags=__future__.annotations.compiler_flag, dont_inherit=True)
    exec(code, ns)
    return ns


def reference_vectors(ns, N, preset):
    """Run the reference host path for one (N, preset); per-record arrays."""
    cs = []
    _, _, cs, _ = ns["gen_constellations"](N, set(), set(), cs, preset)
    m = len(cs)
    soa = ns["TaskSoA"](m)
    w = [0] * m
    soa, w = ns["build_soa_for_range"](N, cs, 0, m, soa, w)
    meta = [(1, 0, 0), (2, 1, 0), (3, 3, 1), (3, 5, 1), (2, 2, 0), (6, 0, 0), (2, 1, 0), (2, 2, 0),
            (0, 4, 1), (4, 4, 1), (5, 4, 1), (7, 4, 1), (13, 0, 0), (14, 1, 0), (14, 5, 1), (14, 2, 0),
            (17, 0, 0), (14, 1, 0), (14, 2, 0), (20, 0, 0), (21, 1, 0), (21, 5, 1), (21, 2, 0),
            (25, 0, 0), (21, 2, 0), (21, 1, 0), (26, 5, 1), (26, 0, 0)]
    n3 = 1 << max(0, N - 3)
    n4 = 1 << max(0, N - 4)
    cat = [3, 0, 0, 0, 4, 0, 3, 3, 0, 0, 0, 0, 3, 0, 0, 4, 0, 3, 3, 3, 0, 0, 4, 0, 3, 3, 0, 3]
    blockK = [n3 if c == 3 else (n4 if c == 4 else 0) for c in cat]
    blockL = [0, 1, 0, 0, 1, 1, 0, 2, 0, 0, 0, 0, 0, 1, 0, 1, 1, 0, 2, 0, 0, 0, 1, 1, 2, 0, 0, 0]
    bm = (1 << N) - 1
    sol = np.zeros(m, np.uint64)
    nodes = np.zeros(m, np.uint64)
    for i in range(m):
        ns["_NODES"][0] = 0
        cnt = ns["dfs_iter"](meta, blockK, blockL, bm, soa.funcid_arr[i], int(soa.ld_arr[i]),
                             int(soa.rd_arr[i]), int(soa.col_arr[i]), soa.row_arr[i], int(soa.free_arr[i]),
                             soa.jmark_arr[i], soa.end_arr[i], soa.mark1_arr[i], soa.mark2_arr[i])
        sol[i] = int(cnt) * int(w[i])
        nodes[i] = ns["_NODES"][0]
    return {
        "startijkl": np.array([c["startijkl"] for c in cs], np.uint64),
        "ld": np.array([c["ld"] for c in cs], np.uint64),
        "rd": np.array([c["rd"] for c in cs], np.uint64),
        "col": np.array([c["col"] for c in cs], np.uint64),
        "solutions": sol,
        "nodes": nodes,
        "fid": np.array(soa.funcid_arr, np.int32),
        "free": np.array(soa.free_arr, np.uint64),
        "ctrl0": np.array(soa.ctrl0_arr, np.uint64),
        "markctrl": np.array(soa.markctrl_arr, np.uint64),
        "task_ld": np.array(soa.ld_arr, np.uint64),
        "task_rd": np.array(soa.rd_arr, np.uint64),
        "task_col": np.array(soa.col_arr, np.uint64),
        "w": np.array(w, np.uint64),
    }


def archive_part():
    digests = {"tasks": {}, "solutions": {}}
    small = {}
    for N in range(6, 22):
        c = np.fromfile(os.path.join(ARCHIVE, f"constellations_N{N}_5.bin"), dtype="<u4").reshape(-1, 4)
        digests["tasks"][str(N)] = {"records": int(c.shape[0]),
                                    "sha256": task_digest(c[:, 3], c[:, 0], c[:, 1], c[:, 2])}
    for N in range(6, 20):
        s = np.fromfile(os.path.join(ARCHIVE, f"solutions_N{N}_5_v2.bin"), dtype="<u8").reshape(-1, 5)
        digests["solutions"][str(N)] = {
            "records": int(s.shape[0]), "sum": int(s[:, 4].sum(dtype=np.uint64)),
            "sha256": solution_digest(s[:, 0], s[:, 1], s[:, 2], s[:, 3], s[:, 4])}
        if N <= 12:
            small[f"N{N}"] = s
    digests["note"] = ("preset 5; tasks: sorted u32 {ld,rd,col,startijkl}; solutions: sorted u64 "
                       "{startijkl,ld,rd,col,solutions}; see golden_util.py")
    with open(os.path.join(HERE, "archive_digests.json"), "w") as f:
        json.dump(digests, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "archive_small.npz"), **small)


def python_part():
    ns = load_reference_host()
    out = {}
    for N in range(6, 13):
        for preset in ((4, 5, 6, 7) if N <= 11 else (4, 5)):
            try:
                v = reference_vectors(ns, N, preset)
            except (ValueError, IndexError):
                continue  # the reference raises on presets too deep for this N
            for k, a in v.items():
                out[f"N{N}_p{preset}_{k}"] = a
    np.savez_compressed(os.path.join(HERE, "ref_py_vectors.npz"), **out)


def c_part():
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", f"REFERENCE_ROOT={REF}"], check=True)
    exe = os.path.join(REPO, "oracle", "_ref", "ref13c")
    txt = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=600).stdout
    totals = {}
    for line in txt.splitlines():
        parts = line.replace(":", " ").split()
        if len(parts) >= 3 and parts[0].isdigit():
            totals[parts[0]] = {"total": int(parts[1]), "status": parts[-1]}
    with open(os.path.join(HERE, "ref_c_totals.json"), "w") as f:
        json.dump({"preset": 4, "source": "10Bit_CUDA/13CUDA_constellation.c", "totals": totals}, f,
                  indent=1, sort_keys=True)


def unique_part():
    spec = importlib.util.spec_from_file_location("ref07", PY07)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    res = {}
    for n in range(4, 12):
        q = mod.NQueens07()
        q.init(n)
        q.NQueens(n)
        res[str(n)] = {"total": q.total, "unique": q.unique}
    with open(os.path.join(HERE, "ref_unique.json"), "w") as f:
        json.dump({"source": "11Bit_Python/07Py_bit_symmetry.py", "values": res}, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    parts = sys.argv[1:] or ["archive", "python", "c", "unique"]
    if "archive" in parts:
        archive_part()
    if "python" in parts:
        python_part()
    if "c" in parts:
        c_part()
    if "unique" in parts:
        unique_part()
    print("golden fixtures written to", HERE)
