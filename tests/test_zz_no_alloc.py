"""The allocation-free entry point nq_exec_solutions_noalloc, through the C ABI.

It exists for callers that must not allocate device memory once running (a
process whose GPU memory belongs to another allocator or a fixed budget, or a
latency-critical loop that cannot afford cudaMalloc's implicit device
synchronisation).  Its counts must equal the regular entry point's, call after
call, although every call reuses the same fixed scratch array.  This file is
collected last so that a failure here comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]

MAX_RECORDS = 131072


def _noalloc(L, N, d_rec, m, start_min, d_sol, d_total, stream):
    return L.nq_exec_solutions_noalloc(N, ctypes.c_void_p(d_rec), m, start_min,
                                       ctypes.c_void_p(d_sol) if d_sol else None, ctypes.c_void_p(d_total),
                                       ctypes.c_void_p(stream))


@pytest.mark.parametrize("N", [10, 13, 16, 17])
def test_noalloc_matches_regular_entry_point_twice(N):
    torch = pytest.importorskip("torch")
    import nqueens
    from nqueens import _lib
    L = _lib.lib()
    eng = nqueens.Engine(0)
    try:
        recs = nqueens.gen_records(N)
        want_total, want_sol = eng.exec_records(N, recs, want_solutions=True)
    finally:
        eng.close()
    m = len(recs)
    assert m <= MAX_RECORDS
    start_min = int((recs["startijkl"] >> 20).min())
    d_rec = torch.from_numpy(recs.view(np.uint8).copy()).cuda()
    d_total = torch.empty(1, dtype=torch.int64, device="cuda")
    d_sol = torch.empty(m, dtype=torch.int64, device="cuda")
    s = torch.cuda.Stream()
    free_after = []
    for call in range(3):   # calls in a row share (and must clear) the same scratch
        d_total.fill_(-1)
        d_sol.fill_(-1)
        torch.cuda.synchronize()
        st = _noalloc(L, N, d_rec.data_ptr(), m, start_min, d_sol.data_ptr(), d_total.data_ptr(), s.cuda_stream)
        assert st == 0, (call, st)
        free_after.append(torch.cuda.mem_get_info()[0])   # the device's free bytes (cudaMemGetInfo)
        assert int(d_total.item()) == want_total, call
        assert np.array_equal(d_sol.cpu().numpy().view(np.uint64), want_sol), call
    # after the first call (which may load the array and kernels), calls take no device memory
    assert free_after[1] == free_after[2] == free_after[0], free_after


def test_noalloc_total_only_and_limits():
    torch = pytest.importorskip("torch")
    import nqueens
    from nqueens import _lib
    L = _lib.lib()
    recs = nqueens.gen_records(12)
    d_rec = torch.from_numpy(recs.view(np.uint8).copy()).cuda()
    d_total = torch.zeros(1, dtype=torch.int64, device="cuda")
    st = _noalloc(L, 12, d_rec.data_ptr(), len(recs), int((recs["startijkl"] >> 20).min()), 0,
                  d_total.data_ptr(), 0)
    assert st == 0 and int(d_total.item()) == 14200
    # beyond the fixed scratch: rejected before any launch, output untouched
    d_total.fill_(7)
    torch.cuda.synchronize()
    st = _noalloc(L, 12, d_rec.data_ptr(), MAX_RECORDS + 1, 3, 0, d_total.data_ptr(), 0)
    assert st == _lib.NQ_EINVAL and int(d_total.item()) == 7
    st = _noalloc(L, 27, d_rec.data_ptr(), 10, 0, 0, d_total.data_ptr(), 0)   # schedule deeper than 24 words
    assert st == _lib.NQ_EINVAL
