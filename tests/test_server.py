"""Serving loop: every request's count is exact and the same alone and in the mix."""
import time

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


def _oracle_answer(oracle_mod, job):
    import nqueens
    if isinstance(job, nqueens.CountJob):
        return oracle_mod.EXPECTED_TOTAL[job.N]
    return oracle_mod.completions(job.N, [r for r, _ in job.queens], [c for _, c in job.queens])


@pytest.mark.parametrize("share_gpu,max_inflight,large_ms", [(True, 3, 0.05), (False, 2, 50.0), (True, 1, 50.0)])
def test_server_results_exact_and_same_as_alone(oracle_mod, share_gpu, max_inflight, large_ms):
    import nqueens
    from nqueens.server import Server, random_completion_queries, run_plain
    jobs = random_completion_queries(60, seed=11, N_range=(8, 13), k_range=(0, 4))
    eng = nqueens.Engine(0)
    try:
        alone = run_plain(eng, jobs)
        with Server(engine=eng, max_inflight=max_inflight, max_batch_jobs=7, share_gpu=share_gpu,
                    large_ms=large_ms) as srv:
            rng = np.random.default_rng(5)
            futs = []
            for j in jobs:                                  # staggered arrivals: batches overlap
                futs.append(srv.submit(j))
                time.sleep(float(rng.exponential(0.0005)))
            srv.drain(120)
            mixed = [f.result(timeout=10) for f in futs]
            st = srv.stats()
        assert mixed == alone
        assert mixed == [_oracle_answer(oracle_mod, j) for j in jobs]
        assert st.completed == len(jobs) and st.batches >= 2
        assert 0 < st.percentile(50) <= st.percentile(99)
    finally:
        eng.close()


def test_server_small_budget_still_exact(oracle_mod):
    """A budget that holds only the largest single request: the bytes in flight never exceed it (requests are
    sized before they are built, so the budget is a hard limit); results stay exact."""
    import nqueens
    from nqueens.server import Server, random_completion_queries
    jobs = random_completion_queries(20, seed=3, N_range=(10, 14), k_range=(1, 3))
    with Server(max_inflight=3, max_batch_jobs=4) as srv:
        srv.budget = max(srv._job_bytes(j) for j in jobs)
        futs = [srv.submit(j) for j in jobs]
        srv.drain(120)
        got = [f.result(timeout=10) for f in futs]
        st = srv.stats()
        assert 0 < st.max_admitted_bytes <= srv.budget
        assert st.batches >= 2
    assert got == [_oracle_answer(oracle_mod, j) for j in jobs]


def test_server_request_beyond_the_budget_fails_alone(oracle_mod):
    """A request whose estimated device bytes exceed the whole budget fails with NQ_ENOMEM and is never
    built; the requests around it are served."""
    import nqueens
    from nqueens.server import Server
    with Server(max_inflight=3, max_batch_jobs=4) as srv:
        small, big = nqueens.CountJob(10), nqueens.CountJob(19)
        srv.budget = srv._job_bytes(small) * 4
        f_small, f_big = srv.submit(small), srv.submit(big)
        srv.drain(120)
        assert f_small.result(timeout=10) == 724
        with pytest.raises(nqueens.NQError) as e:
            f_big.result(timeout=10)
        assert e.value.status == -5


def test_server_rejects_bad_request():
    import nqueens
    from nqueens.server import Server
    with Server(max_inflight=1) as srv:
        with pytest.raises(TypeError):
            srv.submit("N=8")
        f = srv.submit(nqueens.CompletionJob(8, [(0, 0), (0, 0)]))   # the same queen twice: a bad argument
        with pytest.raises(Exception):
            f.result(timeout=30)


def test_batch_resident_blocks_and_shared_grid():
    """A batch reports the resident capacity of its own launch (at least that of the deepest wide stack), and
    a launch on a share of it still counts exactly."""
    import nqueens
    eng = nqueens.Engine(0)
    try:
        b = eng.batch([nqueens.CountJob(14), nqueens.CountJob(12), nqueens.CompletionJob(11, [(0, 3)])])
        full = b.resident_blocks()
        assert b.h2d_bytes >= 16 * 2 and b.device_bytes > b.h2d_bytes
        assert full >= eng.resident_blocks(True, 18) > 0
        want = b.run(use_graph=False)
        b.set_grid(max(1, full // 8))
        assert np.array_equal(b.run(use_graph=False), want)
        assert int(want[0]) == 365596 and int(want[1]) == 14200
        b.close()
    finally:
        eng.close()
