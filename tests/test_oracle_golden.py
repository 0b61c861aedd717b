"""The CPU oracle against the reference's golden vectors (no GPU needed).

Pins: the archived task lists and per-constellation solutions
(13Bit_codon/Archive/bin), the reference's Python host functions run under
CPython (ref_py_vectors.npz), the reference C restatement's totals
(ref_c_totals.json), the symmetry-method unique counts (ref_unique.json) and
the known-answer tables.
"""
import json
import os

import numpy as np
import pytest

from golden_util import canonical_order, solution_digest, task_digest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _json(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.mark.parametrize("N", range(6, 22))
def test_generator_matches_archived_task_lists(oracle_mod, N):
    d = _json("archive_digests.json")["tasks"][str(N)]
    r = oracle_mod.gen_constellations(N, 5)
    assert len(r) == d["records"]
    assert task_digest(r.startijkl, r.ld, r.rd, r.col) == d["sha256"]


@pytest.mark.parametrize("N", range(6, 17))
def test_solver_matches_archived_solutions(oracle_mod, N):
    d = _json("archive_digests.json")["solutions"][str(N)]
    r = oracle_mod.gen_constellations(N, 5)
    sol = oracle_mod.exec_solutions(N, r)
    assert int(sol.sum(dtype=np.uint64)) == d["sum"] == oracle_mod.EXPECTED_TOTAL[N]
    assert solution_digest(r.startijkl, r.ld, r.rd, r.col, sol) == d["sha256"]


@pytest.mark.parametrize("N", range(6, 13))
def test_solver_matches_archived_records(oracle_mod, N):
    """Record-for-record against the raw archived records (not only the digest)."""
    s = np.load(os.path.join(GOLDEN, "archive_small.npz"))[f"N{N}"]
    r = oracle_mod.gen_constellations(N, 5)
    sol = oracle_mod.exec_solutions(N, r, threads=1)
    a = canonical_order(r.startijkl, r.ld, r.rd, r.col)
    b = canonical_order(s[:, 0], s[:, 1], s[:, 2], s[:, 3])
    assert np.array_equal(r.startijkl[a].astype(np.uint64), s[b, 0])
    assert np.array_equal(r.ld[a], s[b, 1]) and np.array_equal(r.rd[a], s[b, 2])
    assert np.array_equal(r.col[a], s[b, 3]) and np.array_equal(sol[a], s[b, 4])


def _ref_py_cases():
    z = np.load(os.path.join(GOLDEN, "ref_py_vectors.npz"))
    return sorted({tuple(k.split("_")[:2]) for k in z.files})


@pytest.mark.parametrize("case", _ref_py_cases())
def test_oracle_matches_reference_python(oracle_mod, case):
    """Generator, weights, counts and node counts equal the reference's own Python code."""
    z = np.load(os.path.join(GOLDEN, "ref_py_vectors.npz"))
    tag = "_".join(case)
    N, preset = int(case[0][1:]), int(case[1][1:])
    ref = {k[len(tag) + 1:]: z[k] for k in z.files if k.startswith(tag + "_")}
    r = oracle_mod.gen_constellations(N, preset)
    assert len(r) == len(ref["startijkl"])
    if len(r) == 0:
        return
    sol, nodes = oracle_mod.exec_solutions(N, r, threads=1, want_nodes=True)
    a = canonical_order(r.startijkl, r.ld, r.rd, r.col)
    b = canonical_order(ref["startijkl"], ref["ld"], ref["rd"], ref["col"])
    for k, v in (("startijkl", r.startijkl), ("ld", r.ld), ("rd", r.rd), ("col", r.col)):
        assert np.array_equal(np.asarray(v, np.uint64)[a], ref[k][b]), k
    assert np.array_equal(sol[a], ref["solutions"][b])
    assert np.array_equal(nodes[a], ref["nodes"][b])


def test_preset_rule(oracle_mod):
    assert [oracle_mod.preset_for(n) for n in (5, 13, 17, 18, 21, 22, 24, 25, 27)] == [5, 5, 5, 6, 6, 7, 7, 8, 8]


@pytest.mark.parametrize("N", range(1, 13))
def test_brute_force_known_answers(oracle_mod, N):
    assert oracle_mod.bit_total(N) == oracle_mod.EXPECTED_TOTAL[N]


@pytest.mark.parametrize("N", range(6, 16))
def test_constellation_totals_dynamic_preset(oracle_mod, N):
    assert oracle_mod.total(N) == oracle_mod.EXPECTED_TOTAL[N]


def test_reference_c_port_totals(oracle_mod):
    """Totals printed by the reference's C restatement agree with the oracle and known answers."""
    d = _json("ref_c_totals.json")["totals"]
    for n, v in d.items():
        N = int(n)
        assert v["total"] == oracle_mod.EXPECTED_TOTAL[N]
        if 6 <= N <= 14:
            assert oracle_mod.total(N, preset=4) == v["total"]


@pytest.mark.parametrize("N", range(4, 13))
def test_unique_symmetry(oracle_mod, N):
    u, t = oracle_mod.unique_symmetry(N)
    assert (u, t) == (oracle_mod.EXPECTED_UNIQUE[N], oracle_mod.EXPECTED_TOTAL[N])
    ref = _json("ref_unique.json")["values"].get(str(N))
    if ref:
        assert (u, t) == (ref["unique"], ref["total"])


@pytest.mark.parametrize("N", range(1, 10))
def test_unique_bruteforce(oracle_mod, N):
    assert oracle_mod.unique_bruteforce(N) == (oracle_mod.EXPECTED_UNIQUE[N], oracle_mod.EXPECTED_TOTAL[N])


def test_completions_bruteforce(oracle_mod):
    # no pre-placed queens: all solutions
    assert oracle_mod.completions(8, [], []) == 92
    # attacking pre-placed queens: none
    assert oracle_mod.completions(8, [0, 1], [0, 1]) == 0
    # every completion with a queen at (0,0) on 8x8 = 4 (known)
    assert oracle_mod.completions(8, [0], [0]) == 4
    # sum over the first row's columns = total
    assert sum(oracle_mod.completions(10, [0], [c]) for c in range(10)) == 724
