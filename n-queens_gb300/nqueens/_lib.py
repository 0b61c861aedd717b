"""ctypes binding of libnqgpu.so (include/nqueens_gb300.h).

The library is the only compute path: if it is missing or cannot be loaded
this module raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnqgpu.so")

NQ_OK = 0
NQ_EINVAL = -1
NQ_ESTACK = -2
NQ_ETIMEOUT = -3
NQ_ECUDA = -4
NQ_ENOMEM = -5
NQ_EPRESET = -6
NQ_EBUSY = -7

NQ_JOB_COUNT = 0
NQ_JOB_COMPLETION = 1

# nq_record: the reference's 16-byte task record (.bin layout)
RECORD_DTYPE = np.dtype([("ld", "<u4"), ("rd", "<u4"), ("col", "<u4"), ("startijkl", "<u4")])


class NQError(RuntimeError):
    """A failed libnqgpu call; .status is the NQ_E* code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


class nq_job(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("N", ctypes.c_int32), ("preset", ctypes.c_int32),
                ("k", ctypes.c_int32), ("rows", ctypes.c_int8 * 8), ("cols", ctypes.c_int8 * 8)]


class nq_record(ctypes.Structure):
    _fields_ = [("ld", ctypes.c_uint32), ("rd", ctypes.c_uint32), ("col", ctypes.c_uint32),
                ("startijkl", ctypes.c_uint32)]


_lib = None

# name -> (restype, argtypes); every symbol include/nqueens_gb300.h declares.
_vp = ctypes.c_void_p
_u64p = ctypes.POINTER(ctypes.c_uint64)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_ip = ctypes.POINTER(ctypes.c_int)
SIGNATURES = {
    "nq_version": (ctypes.c_char_p, []),
    "nq_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "nq_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int]),
    "nq_destroy": (None, [_vp]),
    "nq_last_error": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_size_t]),
    "nq_device_name": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_size_t]),
    "nq_device_sms": (ctypes.c_int, [_vp, _ip]),
    "nq_set_config": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "nq_get_config": (ctypes.c_int, [_vp, _ip, _ip, _ip]),
    "nq_set_queue_order": (ctypes.c_int, [_vp, ctypes.c_int]),
    "nq_get_queue_order": (ctypes.c_int, [_vp, _ip]),
    "nq_preset_for": (ctypes.c_int, [ctypes.c_int]),
    "nq_gen_constellations": (ctypes.c_int64, [ctypes.c_int, ctypes.c_int, _vp, ctypes.c_int64]),
    "nq_gen_constellations_wide": (ctypes.c_int64, [ctypes.c_int, ctypes.c_int, _u64p, _u64p, _u64p, _u32p,
                                                   ctypes.c_int64]),
    "nq_exec_solutions": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int64, _u64p, _u64p]),
    "nq_exec_solutions_device": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int64, ctypes.c_int, _vp, _vp,
                                                _vp]),
    "nq_exec_solutions_noalloc": (ctypes.c_int, [ctypes.c_int, _vp, ctypes.c_int64, ctypes.c_int, _vp, _vp, _vp]),
    "nq_sync": (ctypes.c_int, [_vp]),
    "nq_last_run_info": (ctypes.c_int, [_vp, _ip, ctypes.POINTER(ctypes.c_int64)]),
    "nq_last_kernel_ms": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "nq_count": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _u64p]),
    "nq_start_constellations": (ctypes.c_int64, [ctypes.c_int, _vp, ctypes.c_int64]),
    "nq_gen_constellations_starts": (ctypes.c_int64, [ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, _vp,
                                                     ctypes.c_int64]),
    "nq_count_starts": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, _u64p]),
    "nq_set_chunk_records": (ctypes.c_int, [_vp, ctypes.c_int64]),
    "nq_last_count_info": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "nq_count_unique": (ctypes.c_int, [_vp, ctypes.c_int, _u64p, _u64p]),
    "nq_count_completions": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _ip, _ip, _u64p]),
    "nq_debug_task_schedule": (ctypes.c_int, [ctypes.c_int, nq_record, _u32p, _u32p, _u32p, ctypes.c_int]),
    "nq_debug_completion_tasks": (ctypes.c_int64, [ctypes.c_int, ctypes.c_int, _ip, _ip, ctypes.c_int, _u32p,
                                                  _u32p, _u32p, ctypes.c_int, ctypes.c_int64, _u64p]),
    "nq_int32_peak": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "nq_batch_create": (ctypes.c_int, [_vp, ctypes.POINTER(nq_job), ctypes.c_int, ctypes.POINTER(_vp)]),
    "nq_batch_tasks": (ctypes.c_int64, [_vp]),
    "nq_batch_set_grid": (ctypes.c_int, [_vp, ctypes.c_int]),
    "nq_resident_blocks": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _ip]),
    "nq_batch_resident_blocks": (ctypes.c_int, [_vp, _ip]),
    "nq_tune": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _ip, _ip, ctypes.POINTER(ctypes.c_float)]),
    "nq_batch_device_bytes": (ctypes.c_int64, [_vp]),
    "nq_job_device_bytes": (ctypes.c_int64, [ctypes.POINTER(nq_job), ctypes.c_int, ctypes.c_int]),
    "nq_batch_h2d_bytes": (ctypes.c_int64, [_vp]),
    "nq_batch_run": (ctypes.c_int, [_vp, ctypes.c_int, _u64p]),
    "nq_batch_run_plain": (ctypes.c_int, [_vp, _u64p]),
    "nq_batch_submit": (ctypes.c_int, [_vp, ctypes.c_int]),
    "nq_batch_poll": (ctypes.c_int, [_vp, _u64p, ctypes.c_int64]),
    "nq_batch_destroy": (None, [_vp]),
}


def lib() -> ctypes.CDLL:
    """Load libnqgpu.so (built by n-queens_gb300/build.py); raises if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python n-queens_gb300/build.py` "
                              "(the engine has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def p64(a: np.ndarray):
    return a.ctypes.data_as(_u64p)


def p32(a: np.ndarray):
    return a.ctypes.data_as(_u32p)
