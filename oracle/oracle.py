"""CPU oracle for the constellation N-Queens path -- TEST INFRASTRUCTURE ONLY.

This module is the checker.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py`` (its ``cpu_baseline`` leg and ``--impl reference``) may import it.
The product package never imports it and has no CPU fallback.

It wraps ``oracle/_build/libnqoracle.so`` (a C restatement of the reference's
Python/Codon host code, see ``nq_oracle.c`` for the file:line map) and adds a
few pure-Python restatements for small cases:

* ``gen_constellations`` -- 14Bit_codon_GPU/356Py_savesp_narrow.py:2837-2926
* ``exec_solutions``     -- 356Py_savesp_narrow.py:2579-2610 (CPU branch)
* ``bit_total``          -- 356Py_savesp_narrow.py:5755-5767
* ``unique_symmetry``    -- 11Bit_Python/07Py_bit_symmetry.py:65-200
* ``unique_bruteforce``  -- enumerate every solution and count classes under
  the 8 board symmetries (pure Python, N <= 10)
* ``EXPECTED_TOTAL``     -- the known-answer table of 356Py_savesp_narrow.py:5775
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnqoracle.so")

# Known totals, 356Py_savesp_narrow.py:5775 (index = N).
EXPECTED_TOTAL = [0, 1, 0, 0, 2, 10, 4, 40, 92, 352, 724, 2680, 14200, 73712, 365596, 2279184,
                  14772512, 95815104, 666090624, 4968057848, 39029188884, 314666222712,
                  2691008701644, 24233937684440, 227514171973736, 2207893435808352,
                  22317699616364044, 234907967154122528]
# Known unique counts, README.en:10-35 / 10Bit_CUDA/01CUDA_Bit_Symmetry.cu:27-50 (index = N).
EXPECTED_UNIQUE = [0, 1, 0, 0, 1, 2, 1, 6, 12, 46, 92, 341, 1787, 9233, 45752, 285053, 1846955,
                   11977939, 83263591, 621012754, 4878666808, 39333324973, 336376244042,
                   3029242658210, 28439272956934, 275986683743434]


def build(quiet: bool = True) -> str:
    """Compile the oracle library with the committed Makefile; returns its path."""
    cmd = ["make", "-s", "-C", HERE, "all"]
    subprocess.run(cmd, check=True, capture_output=quiet)
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.orc_gen_constellations.restype = ctypes.c_int64
        L.orc_gen_constellations.argtypes = [ctypes.c_int, ctypes.c_int, u64p, u64p, u64p, u32p, ctypes.c_int64]
        L.orc_exec_solutions.restype = ctypes.c_int
        L.orc_exec_solutions.argtypes = [ctypes.c_int, ctypes.c_int64, u64p, u64p, u64p, u32p, u64p, u64p,
                                         ctypes.c_int]
        L.orc_bit_total.restype = ctypes.c_uint64
        L.orc_bit_total.argtypes = [ctypes.c_int]
        L.orc_completions.restype = ctypes.c_uint64
        L.orc_completions.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_int)]
        L.orc_unique_symmetry.restype = ctypes.c_int
        L.orc_unique_symmetry.argtypes = [ctypes.c_int] + [u64p] * 5
        L.orc_preset_for.restype = ctypes.c_int
        L.orc_preset_for.argtypes = [ctypes.c_int, ctypes.c_int]
        L.orc_symmetry.restype = ctypes.c_int
        L.orc_symmetry.argtypes = [ctypes.c_int, ctypes.c_int]
        L.orc_jasmin.restype = ctypes.c_int
        L.orc_jasmin.argtypes = [ctypes.c_int, ctypes.c_int]
        _lib = L
    return _lib


def _p64(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))


def _p32(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


@dataclass
class Records:
    """Constellation records as the reference produces them (full-width ld/rd/col)."""
    ld: np.ndarray        # uint64
    rd: np.ndarray        # uint64
    col: np.ndarray       # uint64
    startijkl: np.ndarray  # uint32

    def __len__(self) -> int:
        return int(self.startijkl.shape[0])


def preset_for(N: int) -> int:
    """select_dynamic_preset_queens (356Py:5744-5753)."""
    return int(lib().orc_preset_for(N, 5))


def gen_constellations(N: int, preset: int) -> Records:
    L = lib()
    z64 = np.zeros(1, np.uint64)
    z32 = np.zeros(1, np.uint32)
    n = L.orc_gen_constellations(N, preset, _p64(z64), _p64(z64), _p64(z64), _p32(z32), 0)
    if n < 0:
        raise ValueError(f"oracle generator rejected N={N} preset={preset} (status {n})")
    ld = np.zeros(n, np.uint64); rd = np.zeros(n, np.uint64); col = np.zeros(n, np.uint64)
    s = np.zeros(n, np.uint32)
    n2 = L.orc_gen_constellations(N, preset, _p64(ld), _p64(rd), _p64(col), _p32(s), n)
    assert n2 == n
    return Records(ld, rd, col, s)


def exec_solutions(N: int, rec: Records, threads: int = 0, want_nodes: bool = False):
    """Per-record weighted counts (uint64), and per-record dfs_iter nodes when asked."""
    L = lib()
    m = len(rec)
    ld = np.ascontiguousarray(rec.ld, np.uint64); rd = np.ascontiguousarray(rec.rd, np.uint64)
    col = np.ascontiguousarray(rec.col, np.uint64); s = np.ascontiguousarray(rec.startijkl, np.uint32)
    sol = np.zeros(m, np.uint64)
    nodes = np.zeros(m, np.uint64) if want_nodes else None
    if threads <= 0:
        threads = os.cpu_count() or 1
    st = L.orc_exec_solutions(N, m, _p64(ld), _p64(rd), _p64(col), _p32(s), _p64(sol),
                              _p64(nodes) if want_nodes else None, threads)
    if st != 0:
        raise ValueError(f"oracle exec_solutions failed with status {st}")
    return (sol, nodes) if want_nodes else sol


def total(N: int, preset: int | None = None, threads: int = 0) -> int:
    """Total count for N through the constellation path (brute force for N <= 5, as the reference)."""
    if N <= 5:
        return bit_total(N)
    p = preset_for(N) if preset is None else preset
    rec = gen_constellations(N, p)
    sol = exec_solutions(N, rec, threads)
    return int(sol.sum(dtype=np.uint64))


def bit_total(N: int) -> int:
    return int(lib().orc_bit_total(N))


def completions(N: int, rows, cols) -> int:
    k = len(rows)
    r = (ctypes.c_int * max(k, 1))(*rows)
    c = (ctypes.c_int * max(k, 1))(*cols)
    return int(lib().orc_completions(N, k, r, c))


def unique_symmetry(N: int):
    """(unique, total) from the symmetry method of 07Py_bit_symmetry.py (N >= 4)."""
    vals = [ctypes.c_uint64(0) for _ in range(5)]
    st = lib().orc_unique_symmetry(N, *[ctypes.byref(v) for v in vals])
    if st != 0:
        raise ValueError(f"unique_symmetry: N={N} outside 4..31")
    return int(vals[0].value), int(vals[1].value)


def unique_bruteforce(N: int):
    """(unique, total) by enumerating all solutions and canonicalising under D4 (pure Python)."""
    sols = []

    def rec(row, cols, ld, rd, dn):
        if row == N:
            sols.append(tuple(cols))
            return
        avail = ((1 << N) - 1) & ~(ld | rd | dn)
        while avail:
            b = avail & -avail
            avail ^= b
            cols.append(b.bit_length() - 1)
            rec(row + 1, cols, (ld | b) << 1, (rd | b) >> 1, dn | b)
            cols.pop()

    rec(0, [], 0, 0, 0)

    def transforms(p):
        n = len(p)
        out = []
        cur = list(p)
        for _ in range(4):
            # rotate 90: queen (r, c) -> (c, n-1-r)
            nxt = [0] * n
            for r, c in enumerate(cur):
                nxt[c] = n - 1 - r
            cur = nxt
            out.append(tuple(cur))
            out.append(tuple(n - 1 - c for c in cur))
        return out

    classes = set(min(transforms(s)) for s in sols)
    return len(classes), len(sols)
