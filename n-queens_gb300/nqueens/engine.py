"""Python host side of the GB300 N-Queens engine.

Mirrors the reference's constellation-solver interface
(14Bit_codon_GPU/356Py_savesp_narrow.py):

* ``gen_constellations(N, ijkl_list, subconst_cache, constellations,
  preset_queens)`` -- same signature and return tuple as 356Py:2837-2926;
  records are generated by the native host generator.
* ``exec_solutions(N, constellations, use_gpu=True, ...)`` -- same signature
  as 356Py:2228; fills ``c["solutions"]`` with each constellation's count
  times its symmetry weight (the sum is the board total, as the reference's
  ``sum(c['solutions'] for c in constellations if c['solutions'] > 0)``).
* ``select_dynamic_preset_queens`` -- 356Py:5744-5753.

plus array-level calls (``gen_records``, ``Engine.exec_records``) that skip
the per-record Python dicts, batches of many jobs, and completion queries.
Every count runs on the GPU through libnqgpu.so; nothing here counts on the
CPU.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import Dict, Iterable, List, Optional, Sequence, Set, Tuple

import numpy as np

from . import _lib
from ._lib import NQError, RECORD_DTYPE, lib

MAX_N = 27


def _check(status: int, handle=None, what: str = "") -> None:
    if status == _lib.NQ_OK:
        return
    msg = lib().nq_strerror(status).decode()
    if handle is not None:
        buf = ctypes.create_string_buffer(512)
        lib().nq_last_error(handle, buf, 512)
        if buf.value:
            msg = buf.value.decode()
    raise NQError(status, f"{what}: {msg}" if what else msg)


def select_dynamic_preset_queens(N: int, preset_queens: int = 5) -> int:
    """Preset-queen depth per N (356Py:5744-5753); outside 5..27 returns preset_queens."""
    if 5 <= N <= 27:
        return int(lib().nq_preset_for(N))
    return preset_queens


def gen_records(N: int, preset: Optional[int] = None) -> np.ndarray:
    """Constellation records for N as the reference's 16-byte .bin layout (RECORD_DTYPE)."""
    p = select_dynamic_preset_queens(N) if preset is None else int(preset)
    L = lib()
    n = L.nq_gen_constellations(N, p, None, 0)
    if n < 0:
        _check(int(n), what=f"gen_constellations(N={N}, preset={p})")
    out = np.zeros(n, RECORD_DTYPE)
    n2 = L.nq_gen_constellations(N, p, out.ctypes.data_as(ctypes.c_void_p), n)
    if n2 != n:
        raise NQError(_lib.NQ_EINVAL, "generator returned a different count on the second call")
    return out


def start_constellations(N: int) -> np.ndarray:
    """The canonical start constellations of N (packed i<<15|j<<10|k<<5|l, ascending, int32): the
    units nq_count_starts counts, the first stage of gen_constellations (356Py:2837-2880)."""
    L = lib()
    n = L.nq_start_constellations(int(N), None, 0)
    if n < 0:
        _check(int(n), what=f"start_constellations(N={N})")
    out = np.zeros(n, np.int32)
    if L.nq_start_constellations(int(N), out.ctypes.data_as(ctypes.c_void_p), n) != n:
        raise NQError(_lib.NQ_EINVAL, "start list changed between calls")
    return out


def gen_records_starts(N: int, first: int, count: int, preset: Optional[int] = None) -> np.ndarray:
    """Records (RECORD_DTYPE) that start constellations [first, first+count) of start_constellations(N)
    expand into, in gen_records' order: concatenated over a partition of the list they are gen_records(N)."""
    p = select_dynamic_preset_queens(N) if preset is None else int(preset)
    L = lib()
    n = L.nq_gen_constellations_starts(int(N), p, int(first), int(count), None, 0)
    if n < 0:
        _check(int(n), what=f"gen_constellations_starts(N={N}, {first}, {count}, preset={p})")
    out = np.zeros(n, RECORD_DTYPE)
    if n and L.nq_gen_constellations_starts(int(N), p, int(first), int(count), out.ctypes.data_as(ctypes.c_void_p),
                                            n) != n:
        raise NQError(_lib.NQ_EINVAL, "generator returned a different count on the second call")
    return out


def gen_records_wide(N: int, preset: Optional[int] = None) -> Tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """(ld, rd, col, startijkl) with the reference's full-width masks (uint64, uint64, uint64, uint32)."""
    p = select_dynamic_preset_queens(N) if preset is None else int(preset)
    L = lib()
    n = L.nq_gen_constellations_wide(N, p, None, None, None, None, 0)
    if n < 0:
        _check(int(n), what=f"gen_constellations(N={N}, preset={p})")
    ld = np.zeros(n, np.uint64); rd = np.zeros(n, np.uint64); col = np.zeros(n, np.uint64)
    s = np.zeros(n, np.uint32)
    L.nq_gen_constellations_wide(N, p, _lib.p64(ld), _lib.p64(rd), _lib.p64(col), _lib.p32(s), n)
    return ld, rd, col, s


def gen_constellations(N: int, ijkl_list: Optional[Set[int]] = None, subconst_cache: Optional[set] = None,
                       constellations: Optional[List[Dict[str, int]]] = None, preset_queens: int = 5):
    """Drop-in for gen_constellations (356Py:2837-2926).

    Appends {"ld", "rd", "col", "startijkl", "solutions": 0} dicts to
    ``constellations`` and returns (ijkl_list, subconst_cache, constellations,
    preset_queens) like the reference.  ``ijkl_list`` receives the canonical
    start constellations; ``subconst_cache`` is returned cleared (the
    reference clears it per start constellation)."""
    ijkl_list = set() if ijkl_list is None else ijkl_list
    subconst_cache = set() if subconst_cache is None else subconst_cache
    constellations = [] if constellations is None else constellations
    ld, rd, col, s = gen_records_wide(N, preset_queens)
    ijkl_list.update(int(x) for x in np.unique(s & 0xFFFFF))
    subconst_cache.clear()
    constellations.extend({"ld": int(a), "rd": int(b), "col": int(c), "startijkl": int(d), "solutions": 0}
                          for a, b, c, d in zip(ld.tolist(), rd.tolist(), col.tolist(), s.tolist()))
    return ijkl_list, subconst_cache, constellations, preset_queens


def records_from_constellations(constellations: Sequence[Dict[str, int]]) -> np.ndarray:
    """Pack reference constellation dicts into 16-byte records (low 32 bits, as its .bin writer)."""
    m = len(constellations)
    out = np.zeros(m, RECORD_DTYPE)
    if m:
        out["ld"] = np.fromiter((c["ld"] & 0xFFFFFFFF for c in constellations), np.uint32, m)
        out["rd"] = np.fromiter((c["rd"] & 0xFFFFFFFF for c in constellations), np.uint32, m)
        out["col"] = np.fromiter((c["col"] & 0xFFFFFFFF for c in constellations), np.uint32, m)
        out["startijkl"] = np.fromiter((c["startijkl"] & 0xFFFFFFFF for c in constellations), np.uint32, m)
    return out


@dataclass
class Result:
    """Board totals.  ``unique`` is 0 on the constellation path, as the reference prints;
    ``Engine.count_unique`` fills it with the symmetry method."""
    total: int
    unique: int = 0


@dataclass
class CountJob:
    """Whole-board total of N (preset None: select_dynamic_preset_queens)."""
    N: int
    preset: Optional[int] = None


@dataclass
class CompletionJob:
    """Completions of an N x N board holding the given pre-placed (row, col) queens."""
    N: int
    queens: Sequence[Tuple[int, int]] = field(default_factory=tuple)


def _job_struct(j) -> _lib.nq_job:
    s = _lib.nq_job()
    if isinstance(j, CountJob):
        s.kind = _lib.NQ_JOB_COUNT; s.N = int(j.N); s.preset = int(j.preset or 0); s.k = 0
    elif isinstance(j, CompletionJob):
        q = list(j.queens)
        if len(q) > 8:
            raise ValueError("at most 8 pre-placed queens per completion job")
        s.kind = _lib.NQ_JOB_COMPLETION; s.N = int(j.N); s.preset = 0; s.k = len(q)
        for i, (r, c) in enumerate(q):
            s.rows[i] = int(r); s.cols[i] = int(c)
    else:
        raise TypeError(f"unknown job type {type(j).__name__}")
    return s


class Batch:
    """Many jobs whose tasks stay resident on the device; run them in one persistent launch."""

    def __init__(self, engine: "Engine", jobs: Sequence):
        self.engine = engine
        self.jobs = list(jobs)
        arr = (_lib.nq_job * len(self.jobs))(*[_job_struct(j) for j in self.jobs])
        h = ctypes.c_void_p()
        _check(lib().nq_batch_create(engine._h, arr, len(self.jobs), ctypes.byref(h)), engine._h, "batch create")
        self._b = h
        self._totals = np.zeros(len(self.jobs), np.uint64)

    @property
    def tasks(self) -> int:
        return int(lib().nq_batch_tasks(self._b))

    @property
    def device_bytes(self) -> int:
        return int(lib().nq_batch_device_bytes(self._b))

    @property
    def h2d_bytes(self) -> int:
        """Host-to-device bytes copied when the batch was built."""
        return int(lib().nq_batch_h2d_bytes(self._b))

    def resident_blocks(self) -> int:
        """DFS blocks resident on the whole GPU for this batch's launch (what set_grid shares out)."""
        v = ctypes.c_int()
        _check(lib().nq_batch_resident_blocks(self._b, ctypes.byref(v)), self.engine._h, "batch resident_blocks")
        return v.value

    def set_grid(self, grid: int) -> None:
        """Blocks of this batch's persistent launch (0: every resident block of the GPU)."""
        _check(lib().nq_batch_set_grid(self._b, int(grid)), self.engine._h, "batch set_grid")

    def run(self, use_graph: bool = True) -> np.ndarray:
        """All jobs in one persistent launch; per-job uint64 totals."""
        _check(lib().nq_batch_run(self._b, int(use_graph), _lib.p64(self._totals)), self.engine._h, "batch run")
        return self._totals.copy()

    def run_plain(self) -> np.ndarray:
        """One launch and one read-back per job (the plain form)."""
        _check(lib().nq_batch_run_plain(self._b, _lib.p64(self._totals)), self.engine._h, "batch run_plain")
        return self._totals.copy()

    def submit(self, use_graph: bool = True) -> None:
        _check(lib().nq_batch_submit(self._b, int(use_graph)), self.engine._h, "batch submit")

    def poll(self, wait_us: int = 0) -> Optional[np.ndarray]:
        """Totals when the submitted run has finished, else None (after waiting up to wait_us)."""
        st = lib().nq_batch_poll(self._b, _lib.p64(self._totals), int(wait_us))
        if st == _lib.NQ_EBUSY:
            return None
        _check(st, self.engine._h, "batch poll")
        return self._totals.copy()

    def close(self) -> None:
        if getattr(self, "_b", None):
            lib().nq_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_JOB_BYTES: Dict[tuple, int] = {}


def job_device_bytes(job, sms: int, split: int = -1) -> int:
    """Upper estimate of the device bytes a batch holding this one job takes on a GPU with `sms`
    multiprocessors (nq_job_device_bytes: host-side sizing, no device needed).  Whole-board counts are
    cached per (N, preset), since sizing one generates its constellations."""
    key = ("count", job.N, job.preset, sms, split) if isinstance(job, CountJob) else None
    if key is not None and key in _JOB_BYTES:
        return _JOB_BYTES[key]
    s = _job_struct(job)
    n = int(lib().nq_job_device_bytes(ctypes.byref(s), int(sms), int(split)))
    if n < 0:
        _check(n, what=f"job_device_bytes(N={job.N})")
    if key is not None:
        _JOB_BYTES[key] = n
    return n


class Engine:
    """One CUDA device and stream of libnqgpu.so."""

    def __init__(self, device: int = 0, block: int = 64, grid: int = 0, split: int = -1, auto_tune: bool = True):
        """auto_tune: when nqueens/tuning.json holds a table for this GPU, each count of an N in
        the table uses its tuned block, grid and split depth (explicit set_config turns this off)."""
        h = ctypes.c_void_p()
        _check(lib().nq_create(ctypes.byref(h), int(device)), what=f"nq_create(device={device})")
        self._h = h
        self.device = device
        self._tuning = None
        self.set_config(block, grid, split)
        if auto_tune and (block, grid, split) == (64, 0, -1):
            from . import tune
            self._tuning = tune.load(self.device_name())

    def device_name(self) -> str:
        buf = ctypes.create_string_buffer(256)
        _check(lib().nq_device_name(self._h, buf, 256), self._h, "device_name")
        return buf.value.decode()

    def _apply_tuning(self, N: int) -> None:
        """The tuned configuration of N, or the defaults (64 threads, one wave, automatic split) for an N
        the table does not hold, so no count inherits the previous N's settings."""
        if self._tuning:
            t = self._tuning.get(str(N), {"block": 64, "grid": 0, "split": -1})
            _check(lib().nq_set_config(self._h, int(t["block"]), int(t["grid"]), int(t["split"])), self._h)

    # -- configuration ---------------------------------------------------
    def set_config(self, block: int = 64, grid: int = 0, split: int = -1) -> None:
        """Threads per block (64/128/256), grid (0: one wave of resident blocks) and split depth
        (-1: automatic, 0..3: expand every task that many levels before the DFS).  Turns the
        autotuned per-N configuration off."""
        _check(lib().nq_set_config(self._h, block, grid, split), self._h, "set_config")
        self._tuning = None

    def tune_native(self, N: int, repeats: int = 2) -> Tuple[int, int, float]:
        """The C ABI's autotuner (nq_tune): (block, split depth, best ms); the handle keeps that configuration
        (and the per-N table is switched off, as with set_config)."""
        b, s, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        _check(lib().nq_tune(self._h, int(N), int(repeats), ctypes.byref(b), ctypes.byref(s), ctypes.byref(ms)),
               self._h, f"tune(N={N})")
        self._tuning = None
        return b.value, s.value, ms.value

    def set_queue_order(self, mode: int) -> None:
        """DFS queue order of single-N counts: 0 generator order, 1 largest estimated subtree first."""
        _check(lib().nq_set_queue_order(self._h, int(mode)), self._h, "set_queue_order")

    def get_queue_order(self) -> int:
        v = ctypes.c_int()
        _check(lib().nq_get_queue_order(self._h, ctypes.byref(v)), self._h, "get_queue_order")
        return v.value

    def get_config(self) -> Tuple[int, int, int]:
        b, g, o = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().nq_get_config(self._h, ctypes.byref(b), ctypes.byref(g), ctypes.byref(o)), self._h)
        return b.value, g.value, o.value

    # -- constellation path ----------------------------------------------
    def exec_records(self, N: int, records: np.ndarray, want_solutions: bool = False):
        """Count host records; returns (total, per-record weighted counts or None)."""
        rec = np.ascontiguousarray(records, RECORD_DTYPE)
        m = int(rec.shape[0])
        self._apply_tuning(N)
        total = np.zeros(1, np.uint64)
        sol = np.zeros(m, np.uint64) if want_solutions else None
        _check(lib().nq_exec_solutions(self._h, int(N), rec.ctypes.data_as(ctypes.c_void_p), m,
                                       _lib.p64(sol) if sol is not None else None, _lib.p64(total)),
               self._h, f"exec_solutions(N={N})")
        return int(total[0]), sol

    def exec_device(self, N: int, d_records: int, m: int, start_min: int, d_total: int,
                    d_solutions: int = 0, stream: int = 0) -> None:
        """Asynchronous count of device-resident records (raw device pointers); see sync()."""
        self._apply_tuning(N)
        _check(lib().nq_exec_solutions_device(self._h, int(N), ctypes.c_void_p(d_records), int(m), int(start_min),
                                              ctypes.c_void_p(d_solutions or None), ctypes.c_void_p(d_total),
                                              ctypes.c_void_p(stream or None)), self._h, f"exec_device(N={N})")

    def sync(self) -> None:
        _check(lib().nq_sync(self._h), self._h, "sync")

    def int32_peak(self, kind: int = 0) -> float:
        """Measured INT32 thread-instructions/s (0 lop3, 1 add, 2 shf, 3 mix)."""
        v = ctypes.c_double()
        _check(lib().nq_int32_peak(self._h, int(kind), ctypes.byref(v)), self._h, "int32_peak")
        return v.value

    def last_run_info(self) -> Tuple[int, int]:
        """(split depth, DFS queue length) of the last exec call."""
        d, q = ctypes.c_int(), ctypes.c_int64()
        _check(lib().nq_last_run_info(self._h, ctypes.byref(d), ctypes.byref(q)), self._h, "last_run_info")
        return d.value, q.value

    def last_kernel_ms(self) -> Tuple[float, float]:
        """(prepare_ms, dfs_ms) of the last exec call, from CUDA events on its stream."""
        a, b = ctypes.c_float(), ctypes.c_float()
        _check(lib().nq_last_kernel_ms(self._h, ctypes.byref(a), ctypes.byref(b)), self._h, "last_kernel_ms")
        return a.value, b.value

    def count(self, N: int, preset: Optional[int] = None) -> Result:
        """Whole-board total (constellation path for N >= 6, GPU brute force for N <= 5)."""
        t = np.zeros(1, np.uint64)
        self._apply_tuning(N)
        _check(lib().nq_count(self._h, int(N), int(preset or 0), _lib.p64(t)), self._h, f"count(N={N})")
        return Result(total=int(t[0]))

    def count_starts(self, N: int, first: int, count: int, preset: Optional[int] = None) -> int:
        """The part of count(N, preset) that comes from start constellations [first, first+count)
        of start_constellations(N); totals over a partition of the list add up to count(N)."""
        t = np.zeros(1, np.uint64)
        self._apply_tuning(N)
        _check(lib().nq_count_starts(self._h, int(N), int(preset or 0), int(first), int(count), _lib.p64(t)),
               self._h, f"count_starts(N={N}, {first}, {count})")
        return int(t[0])

    def set_chunk_records(self, records: int) -> None:
        """Records per chunk of count() (0: the library default); bounds the host memory of large boards."""
        _check(lib().nq_set_chunk_records(self._h, int(records)), self._h, "set_chunk_records")

    def last_count_info(self) -> Tuple[int, int]:
        """(chunks, records) of the last count()."""
        c, r = ctypes.c_int64(), ctypes.c_int64()
        _check(lib().nq_last_count_info(self._h, ctypes.byref(c), ctypes.byref(r)), self._h, "last_count_info")
        return c.value, r.value

    def count_unique(self, N: int) -> Result:
        """Unique and total counts by the symmetry method (07Py_bit_symmetry.py), 4 <= N <= 27."""
        u = np.zeros(1, np.uint64)
        t = np.zeros(1, np.uint64)
        _check(lib().nq_count_unique(self._h, int(N), _lib.p64(u), _lib.p64(t)), self._h, f"count_unique(N={N})")
        return Result(total=int(t[0]), unique=int(u[0]))

    def count_completions(self, N: int, queens: Sequence[Tuple[int, int]]) -> int:
        """Number of full placements containing the pre-placed (row, col) queens."""
        q = list(queens)
        rows = (ctypes.c_int * max(1, len(q)))(*[int(r) for r, _ in q])
        cols = (ctypes.c_int * max(1, len(q)))(*[int(c) for _, c in q])
        t = np.zeros(1, np.uint64)
        _check(lib().nq_count_completions(self._h, int(N), len(q), rows, cols, _lib.p64(t)), self._h,
               f"count_completions(N={N})")
        return int(t[0])

    def resident_blocks(self, wide: bool = True, maxt: int = 18) -> int:
        """DFS blocks resident on the whole GPU at this block size and stack depth."""
        v = ctypes.c_int()
        _check(lib().nq_resident_blocks(self._h, int(wide), int(maxt), ctypes.byref(v)), self._h, "resident_blocks")
        return v.value

    def sms(self) -> int:
        v = ctypes.c_int()
        _check(lib().nq_device_sms(self._h, ctypes.byref(v)), self._h, "device_sms")
        return v.value

    def job_device_bytes(self, job) -> int:
        """Upper estimate of the device bytes a batch of this one job takes on this GPU (nq_job_device_bytes)."""
        return job_device_bytes(job, self.sms(), self.get_config()[2])

    def batch(self, jobs: Iterable) -> Batch:
        return Batch(self, list(jobs))

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().nq_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default: Optional[Engine] = None


def default_engine() -> Engine:
    """The process's engine: device LOCAL_RANK under a per-GPU launcher (torchrun), device 0 otherwise or
    when the launcher gives each rank only its own device."""
    global _default
    if _default is None:
        dev = int(os.environ.get("LOCAL_RANK", "0"))
        try:
            _default = Engine(dev)
        except NQError:
            if dev == 0:
                raise
            _default = Engine(0)
    return _default


def exec_solutions(N: int, constellations: List[Dict[str, int]], use_gpu: bool = True, gpu_block: int = 64,
                   gpu_max_blocks: int = 0, gpu_log_level: int = 0, gpu_sort_mode: int = -1, **_ignored) -> None:
    """Drop-in for exec_solutions (356Py:2228-2610), GPU branch.

    Writes c["solutions"] = count x symmetry weight for every constellation.
    gpu_block selects threads per block (64/128/256) and gpu_max_blocks the
    grid (0: one wave of resident blocks); the reference's reorder knobs
    (gpu_sort_mode and the rest) are accepted and ignored, since the queue is
    balanced by splitting.  use_gpu=False is rejected: this engine has no CPU
    path."""
    if not use_gpu:
        raise ValueError("the GB300 engine has no CPU path (use_gpu=False is the reference's own CPU branch)")
    if not constellations:
        return
    eng = default_engine()
    block = gpu_block if gpu_block in (64, 128, 256) else 64
    if (block, int(gpu_max_blocks)) != (64, 0):      # explicit launch knobs; the defaults keep the tuned table
        _, _, split = eng.get_config()
        eng.set_config(block, max(0, int(gpu_max_blocks)), split)
    recs = records_from_constellations(constellations)
    total, sol = eng.exec_records(N, recs, want_solutions=True)
    for c, v in zip(constellations, sol.tolist()):     # tolist() gives Python ints
        c["solutions"] = v
    if gpu_log_level >= 1:
        print(f"[gpu-summary] N={N} constellations={len(constellations)} total={total}")


def count(N: int, preset: Optional[int] = None, unique: bool = False) -> Result:
    """Whole-board total for N on the default engine (device 0).  With unique=True
    both counts come from the symmetry method (N >= 4)."""
    if unique:
        return default_engine().count_unique(N)
    return default_engine().count(N, preset)
