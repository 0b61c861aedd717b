"""The reference's on-disk task and solution formats.

* Task list ``constellations_N{N}_{P}.bin``: 16-byte little-endian records
  ``{ld, rd, col, startijkl}`` as u32 (writer: ``append_constellations_bin``,
  14Bit_codon_GPU/356Py_savesp_narrow.py:2981-2986; size check
  ``validate_bin_file`` :2941-2948), with a ``.done`` sidecar holding the
  record count of a complete file (:2961-2979, :3086-3102).
* Solution cache v2 ``solutions_N{N}_{P}_v2.bin``: 40-byte little-endian u64
  records ``{startijkl, ld, rd, col, solutions}`` (writer
  ``save_solutions_bin_v2``, 13Bit_codon/18Py_constellations_GPU_cuda_codon.py:
  1841-1855; loader keyed by ``(startijkl, ld, rd, col)``, :1896-1927).

These files let the engine consume the reference's cached task lists and write
solution files the reference can load.  Corrupt inputs raise ``FormatError``.

``stream_tasks`` writes a task list the way the reference's streamed writer does
(``gen_constellations_stream_to_bin``, 356Py:2988-3084): the file is truncated
and its ``.done`` set to 0, the records of a block of start constellations at a
time are appended, and ``.done`` gets the record count only once the file is
complete, so host memory stays bounded by one block at the largest boards.
``ensure_tasks`` is its cache check (``ensure_constellations_bin_stream``,
:3086-3102): a file whose ``.done`` matches its size is reused, any other is
rebuilt.
"""
from __future__ import annotations

import os
from typing import Dict, List, Optional, Tuple

import numpy as np

from ._lib import RECORD_DTYPE

SOLUTION_DTYPE = np.dtype([("startijkl", "<u8"), ("ld", "<u8"), ("rd", "<u8"), ("col", "<u8"),
                           ("solutions", "<u8")])


class FormatError(ValueError):
    """A task or solution file that is truncated, mis-sized or incomplete."""


def task_file_name(N: int, preset: int) -> str:
    return f"constellations_N{N}_{preset}.bin"


def solution_file_name(N: int, preset: int, tag: str = "") -> str:
    return f"solutions_N{N}_{preset}{'_' + tag if tag else ''}_v2.bin"


def read_done(path: str) -> int:
    """Record count in a ``.done`` sidecar, -1 when absent or unreadable (356Py:2961-2969)."""
    try:
        with open(path) as f:
            text = f.read().strip()
        return int(text) if text else -1
    except (OSError, ValueError):
        return -1


def write_done(path: str, count: int) -> None:
    with open(path, "w") as f:
        f.write(f"{int(count)}\n")


def load_tasks(path: str, require_done: bool = False) -> np.ndarray:
    """Read a 16-byte-record task list (RECORD_DTYPE).  With require_done the
    ``.done`` sidecar must exist and match the record count (a complete file)."""
    size = os.path.getsize(path)
    if size % 16 != 0:
        raise FormatError(f"{path}: size {size} is not a multiple of 16 bytes")
    recs = np.fromfile(path, dtype=RECORD_DTYPE)
    if require_done:
        done = read_done(path + ".done")
        if done != len(recs):
            raise FormatError(f"{path}: .done records {done} != file records {len(recs)} (incomplete write)")
    return recs


def save_tasks(path: str, records: np.ndarray, write_sidecar: bool = True) -> None:
    """Write records (RECORD_DTYPE) then the ``.done`` sidecar, as the reference's streaming writer."""
    rec = np.ascontiguousarray(records, RECORD_DTYPE)
    tmp = path + ".tmp"
    rec.tofile(tmp)
    os.replace(tmp, path)
    if write_sidecar:
        write_done(path + ".done", len(rec))


def load_solutions(path: str) -> np.ndarray:
    size = os.path.getsize(path)
    if size == 0 or size % 40 != 0:
        raise FormatError(f"{path}: size {size} is not a positive multiple of 40 bytes")
    return np.fromfile(path, dtype=SOLUTION_DTYPE)


def save_solutions(path: str, ld, rd, col, startijkl, solutions) -> None:
    """Write the 40-byte v2 solution records (full-width masks, as the reference's Python ints)."""
    out = np.zeros(len(solutions), SOLUTION_DTYPE)
    out["startijkl"] = np.asarray(startijkl, np.uint64)
    out["ld"] = np.asarray(ld, np.uint64)
    out["rd"] = np.asarray(rd, np.uint64)
    out["col"] = np.asarray(col, np.uint64)
    out["solutions"] = np.asarray(solutions, np.uint64)
    tmp = path + ".tmp"
    out.tofile(tmp)
    os.replace(tmp, path)


def solutions_lookup(sol: np.ndarray) -> Dict[Tuple[int, int, int, int], int]:
    """Key (startijkl, ld, rd, col) -> solutions, the reference loader's map (18Py:1919-1925)."""
    return {(int(r["startijkl"]), int(r["ld"]), int(r["rd"]), int(r["col"])): int(r["solutions"]) for r in sol}


def fill_from_solutions(constellations: List[dict], sol: np.ndarray) -> Optional[Tuple[int, int, int, int]]:
    """Fill c["solutions"] from a v2 file; returns the first missing key (a cache miss) or None."""
    mp = solutions_lookup(sol)
    for c in constellations:
        key = (int(c["startijkl"]), int(c["ld"]), int(c["rd"]), int(c["col"]))
        if key not in mp:
            return key
        c["solutions"] = mp[key]
    return None


def stream_tasks(path: str, N: int, preset: Optional[int] = None, starts_per_block: int = 256) -> int:
    """Write the task list of N (preset None: the dynamic preset) to path block by block of start
    constellations; returns the record count.  The file's bytes equal save_tasks(path, gen_records(N))."""
    from .engine import gen_records_starts, start_constellations
    if starts_per_block < 1:
        raise ValueError("starts_per_block must be >= 1")
    n_starts = len(start_constellations(N))
    with open(path, "wb"):
        pass
    write_done(path + ".done", 0)
    total = 0
    with open(path, "ab") as f:
        for a in range(0, n_starts, starts_per_block):
            recs = gen_records_starts(N, a, min(starts_per_block, n_starts - a), preset)
            recs.tofile(f)
            total += len(recs)
        f.flush()
        os.fsync(f.fileno())
    write_done(path + ".done", total)
    return total


def ensure_tasks(N: int, preset: Optional[int] = None, directory: str = ".", starts_per_block: int = 256) -> str:
    """Path of a complete task file constellations_N{N}_{P}.bin in directory, written by stream_tasks
    unless a complete one (``.done`` equal to its record count) is already there."""
    from .engine import select_dynamic_preset_queens
    p = select_dynamic_preset_queens(N) if preset is None else int(preset)
    path = os.path.join(directory, task_file_name(N, p))
    size = os.path.getsize(path) if os.path.exists(path) else -1
    if size > 0 and size % 16 == 0 and read_done(path + ".done") == size // 16:
        return path
    stream_tasks(path, N, p, starts_per_block)
    return path
