"""Chunked counting with a progress file, so a long count can resume.

The reference's restart unit is the chunk (``chunk_only`` / ``debug_chunk_start``
/ ``chunk_list_spec``, 14Bit_codon_GPU/356Py_savesp_narrow.py:2418-2435 and
:5539-5550) with a per-chunk progress TSV (:3330-3338).  Here the task list is
cut into fixed chunks; after each chunk one line ``chunk<TAB>first<TAB>end<TAB>total``
is appended to the progress file and flushed, and a rerun skips the chunks
already recorded.  The file starts with a header naming N, the record count and
a digest of the records, so a progress file never resumes a different task list.

``count_resumable`` does the same for a whole-board count without holding the
task list: its chunks are ranges of the board's start constellations, each
generated and counted on the GPU by ``Engine.count_starts`` (host memory stays
bounded), so a count longer than one sitting -- N=24 and up -- is spread over
several runs that share the progress file.
"""
from __future__ import annotations

import hashlib
import os
import time
from typing import Callable, Dict, Optional

import numpy as np

from ._lib import RECORD_DTYPE
from .engine import select_dynamic_preset_queens, start_constellations


def _digest(records: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(records, RECORD_DTYPE).tobytes()).hexdigest()[:32]


def _header(N: int, records: np.ndarray, chunk: int) -> str:
    return f"# nqueens progress N={N} records={len(records)} chunk={chunk} sha256={_digest(records)}\n"


def read_progress(path: str, header: str) -> Dict[int, int]:
    """Chunk index -> total from a progress file written for the same task list."""
    if not os.path.exists(path):
        return {}
    done: Dict[int, int] = {}
    with open(path) as f:
        first = f.readline()
        if first != header:
            raise ValueError(f"{path} belongs to another task list or chunk size")
        for line in f:
            parts = line.rstrip("\n").split("\t")
            if len(parts) != 4:
                break                      # a torn last line from an interrupted write: redo that chunk
            done[int(parts[0])] = int(parts[3])
    return done


def exec_records_resumable(counter: Callable[[int, np.ndarray], int], N: int, records: np.ndarray,
                           progress_path: str, chunk: int = 1 << 20,
                           stop_after: Optional[int] = None) -> Optional[int]:
    """Total over all chunks, resuming from progress_path.  ``counter(N, recs) -> total``
    counts one chunk (an Engine's exec_records, for instance).  ``stop_after`` returns None
    after that many newly counted chunks (an interruption, for tests)."""
    rec = np.ascontiguousarray(records, RECORD_DTYPE)
    header = _header(N, rec, chunk)
    done = read_progress(progress_path, header)
    if not os.path.exists(progress_path):
        with open(progress_path, "w") as f:
            f.write(header)
    n_chunks = (len(rec) + chunk - 1) // chunk
    counted = 0
    with open(progress_path, "a") as f:
        for c in range(n_chunks):
            if c in done:
                continue
            if stop_after is not None and counted >= stop_after:
                return None
            a, b = c * chunk, min(len(rec), (c + 1) * chunk)
            t = int(counter(N, rec[a:b]))
            f.write(f"{c}\t{a}\t{b}\t{t}\n")
            f.flush()
            os.fsync(f.fileno())
            done[c] = t
            counted += 1
    return sum(done[c] for c in range(n_chunks))


def _starts_header(N: int, preset: int, starts: np.ndarray, chunk: int) -> str:
    d = hashlib.sha256(np.ascontiguousarray(starts, np.int32).tobytes()).hexdigest()[:32]
    return f"# nqueens progress N={N} preset={preset} starts={len(starts)} chunk={chunk} sha256={d}\n"


def count_resumable(eng, N: int, progress_path: str, preset: Optional[int] = None, chunk: int = 64,
                    stop_after: Optional[int] = None, log: Optional[Callable[[str], None]] = None,
                    time_limit: Optional[float] = None) -> Optional[int]:
    """Whole-board total of N, counted in chunks of ``chunk`` start constellations with
    ``eng.count_starts`` and resumed from progress_path.  Returns None, leaving the rest for a later
    run, after ``stop_after`` newly counted chunks, or when ``time_limit`` seconds would be passed:
    no chunk starts unless 1.5 x the longest chunk of this run still fits."""
    p = select_dynamic_preset_queens(N) if preset is None else int(preset)
    starts = start_constellations(N)
    header = _starts_header(N, p, starts, chunk)
    done = read_progress(progress_path, header)
    if not os.path.exists(progress_path):
        with open(progress_path, "w") as f:
            f.write(header)
    n_chunks = (len(starts) + chunk - 1) // chunk
    counted = 0
    t_start = time.monotonic()
    longest = 0.0
    with open(progress_path, "a") as f:
        for c in range(n_chunks):
            if c in done:
                continue
            if stop_after is not None and counted >= stop_after:
                return None
            if time_limit is not None and time.monotonic() - t_start + 1.5 * longest > time_limit:
                return None
            a, b = c * chunk, min(len(starts), (c + 1) * chunk)
            t0 = time.monotonic()
            t = eng.count_starts(N, a, b - a, p)
            longest = max(longest, time.monotonic() - t0)
            f.write(f"{c}\t{a}\t{b}\t{t}\n")
            f.flush()
            os.fsync(f.fileno())
            done[c] = t
            counted += 1
            if log:
                log(f"N={N} chunk {c + 1}/{n_chunks} starts [{a}, {b}) total {t} {time.monotonic() - t0:.1f} s")
    return sum(done[c] for c in range(n_chunks))
