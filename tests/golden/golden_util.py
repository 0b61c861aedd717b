"""Canonical forms and digests shared by make_golden.py and the parity tests.

Record order is not part of any result (the reference iterates a Python set),
so every comparison sorts records by the key (startijkl, ld, rd, col), the key
the reference's own solution-cache loader uses
(13Bit_codon/18Py_constellations_GPU_cuda_codon.py:1919-1925).
"""
from __future__ import annotations

import hashlib

import numpy as np


def canonical_order(startijkl, ld, rd, col) -> np.ndarray:
    """Index array that sorts records by (startijkl, ld, rd, col)."""
    keys = [np.asarray(col, np.uint64), np.asarray(rd, np.uint64), np.asarray(ld, np.uint64),
            np.asarray(startijkl, np.uint64)]
    return np.lexsort(keys)


def task_digest(startijkl, ld, rd, col) -> str:
    """sha256 of the sorted 16-byte task records {ld, rd, col, startijkl} as u32 LE.

    ld/rd/col are truncated to 32 bits, as the reference's .bin writer does
    (356Py_savesp_narrow.py:2931-2986)."""
    s = np.asarray(startijkl, np.uint64)
    l32 = np.asarray(ld, np.uint64) & 0xFFFFFFFF
    r32 = np.asarray(rd, np.uint64) & 0xFFFFFFFF
    c32 = np.asarray(col, np.uint64) & 0xFFFFFFFF
    o = canonical_order(s, l32, r32, c32)
    arr = np.stack([l32[o], r32[o], c32[o], s[o]], 1).astype("<u4")
    return hashlib.sha256(arr.tobytes()).hexdigest()


def solution_digest(startijkl, ld, rd, col, solutions) -> str:
    """sha256 of the sorted 40-byte solution records {startijkl, ld, rd, col, solutions} as u64 LE
    (the solutions-v2 layout, 18Py_constellations_GPU_cuda_codon.py:1841-1855)."""
    s = np.asarray(startijkl, np.uint64)
    l = np.asarray(ld, np.uint64)
    r = np.asarray(rd, np.uint64)
    c = np.asarray(col, np.uint64)
    v = np.asarray(solutions, np.uint64)
    o = canonical_order(s, l, r, c)
    arr = np.stack([s[o], l[o], r[o], c[o], v[o]], 1).astype("<u8")
    return hashlib.sha256(arr.tobytes()).hexdigest()
