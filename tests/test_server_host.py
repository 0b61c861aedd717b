"""Serving loop host logic on the CPU: lanes, admission by budget, failure isolation, drain timeout.

The server's batches are replaced by a fake that answers from the oracle after a delay, so the scheduling code
runs exactly as on a GPU machine while nothing touches a device.
"""
import threading
import time

import numpy as np
import pytest

import nqueens
from nqueens import server as srv_mod
from nqueens._lib import NQError


class FakeBatch:
    """Stands in for engine.Batch: same calls, answers from the oracle, finishes `delay_s` after submit."""
    created = []
    delay_s = 0.01
    never_finish = False
    bytes_per_job = 1 << 20
    lock = threading.Lock()

    def __init__(self, engine, jobs):
        import oracle
        for j in jobs:
            if isinstance(j, nqueens.CompletionJob) and any(not (0 <= r < j.N and 0 <= c < j.N) for r, c in j.queens):
                raise NQError(-1, "batch job: bad pre-placed queens")
        self.jobs = list(jobs)
        self.device_bytes = FakeBatch.bytes_per_job * len(jobs)
        self.h2d_bytes = 16 * len(jobs)
        self.grid = None
        self.t_submit = None
        self.answers = []
        for j in jobs:
            if isinstance(j, nqueens.CountJob):
                self.answers.append(oracle.EXPECTED_TOTAL[j.N])
            else:
                self.answers.append(oracle.completions(j.N, [r for r, _ in j.queens], [c for _, c in j.queens]))
        with FakeBatch.lock:
            FakeBatch.created.append(self)

    def resident_blocks(self):
        return 1216

    def set_grid(self, grid):
        self.grid = grid

    def submit(self, use_graph=True):
        self.t_submit = time.perf_counter()

    def poll(self, wait_us=0):
        if FakeBatch.never_finish or time.perf_counter() - self.t_submit < FakeBatch.delay_s:
            return None
        return np.array(self.answers, np.uint64)

    def close(self):
        pass


class FakeEngine:
    """Stands in for engine.Engine in the server: the host-side sizing call only."""

    def __init__(self, real_sizing=False):
        self.real_sizing = real_sizing

    def job_device_bytes(self, job):
        if self.real_sizing:                 # the library's host-side sizing, as on a GB300 (152 SMs)
            return nqueens.engine.job_device_bytes(job, 152)
        return FakeBatch.bytes_per_job


@pytest.fixture
def fake(monkeypatch, oracle_mod):
    FakeBatch.created = []
    FakeBatch.delay_s = 0.01
    FakeBatch.never_finish = False
    FakeBatch.bytes_per_job = 1 << 20
    monkeypatch.setattr(srv_mod, "Batch", FakeBatch)
    return FakeBatch


def _serve(jobs, **kw):
    with srv_mod.Server(engine=FakeEngine(), poll_us=100, **kw) as s:
        futs = [s.submit(j) for j in jobs]
        s.drain(60)
        return [f.result() for f in futs], s.stats()


def test_results_in_submission_order(fake, oracle_mod):
    jobs = srv_mod.random_completion_queries(40, seed=3, N_range=(6, 11), k_range=(0, 3))
    got, st = _serve(jobs, max_batch_jobs=5)
    want = [oracle_mod.EXPECTED_TOTAL[j.N] if isinstance(j, nqueens.CountJob) else
            oracle_mod.completions(j.N, [r for r, _ in j.queens], [c for _, c in j.queens]) for j in jobs]
    assert got == want
    assert st.completed == len(jobs) and len(st.latencies_by_request) == len(jobs)
    assert st.h2d_bytes == 16 * len(jobs) and st.d2h_bytes == 8 * len(jobs)
    assert all(len(b.jobs) <= 5 for b in fake.created)


def test_large_requests_get_a_batch_each_and_the_large_share(fake):
    fake.delay_s = 0.3
    jobs = [nqueens.CountJob(20), nqueens.CountJob(8), nqueens.CountJob(19), nqueens.CountJob(9)]
    _serve(jobs, large_ms=50.0, large_share=0.75)
    large = [b for b in fake.created if any(isinstance(j, nqueens.CountJob) and j.N >= 19 for j in b.jobs)]
    assert len(large) == 2 and all(len(b.jobs) == 1 for b in large)
    assert all(b.grid == 912 for b in large)                       # 0.75 of 1216 resident blocks
    small = [b for b in fake.created if b not in large]
    assert small and all(b.grid == 304 for b in small)             # the other 0.25, beside a large batch


def test_small_batches_take_the_whole_gpu_when_no_large_batch_runs(fake):
    _serve([nqueens.CountJob(8), nqueens.CountJob(9)], large_ms=50.0, large_share=0.75)
    assert fake.created and all(b.grid == 1216 for b in fake.created)


def test_budget_holds_batches_until_memory_returns(fake):
    fake.bytes_per_job = 1 << 30               # each built batch takes more than the whole budget
    jobs = [nqueens.CountJob(n) for n in (6, 7, 8, 9, 10, 11)]
    got, st = _serve(jobs, budget_bytes=1 << 30, max_batch_jobs=4, max_inflight=3)
    assert got == [4, 40, 92, 352, 724, 2680]
    assert st.max_inflight_seen == 1 and st.batches == len(fake.created) >= 2


def test_batches_overlap_within_the_budget(fake):
    fake.delay_s = 0.2
    jobs = [nqueens.CountJob(n) for n in (6, 7, 8, 9, 10, 11)]
    got, st = _serve(jobs, budget_bytes=1 << 34, max_batch_jobs=3, max_inflight=3)
    assert got == [4, 40, 92, 352, 724, 2680]
    assert st.max_inflight_seen >= 2


def test_bad_request_fails_alone(fake):
    jobs = [nqueens.CountJob(8), nqueens.CompletionJob(8, [(9, 0)]), nqueens.CountJob(10)]
    with srv_mod.Server(engine=FakeEngine(), poll_us=100, max_batch_jobs=8) as s:
        futs = [s.submit(j) for j in jobs]
        s.drain(60)
        assert futs[0].result() == 92 and futs[2].result() == 724
        with pytest.raises(NQError):
            futs[1].result()


def test_drain_times_out_when_a_batch_never_finishes(fake):
    fake.never_finish = True
    s = srv_mod.Server(engine=FakeEngine(), poll_us=100)
    try:
        s.submit(nqueens.CountJob(8))
        with pytest.raises(TimeoutError):
            s.drain(0.3)
    finally:
        fake.never_finish = False
        s.close()


def test_submit_rejects_other_objects(fake):
    with srv_mod.Server(engine=FakeEngine(), poll_us=100) as s:
        with pytest.raises(TypeError):
            s.submit((8, []))


def test_request_larger_than_the_budget_fails_alone(fake):
    """Admission sizes each request before building it (nq_job_device_bytes): a whole N=22 board
    (28.7 M records at preset 7, several GB) cannot fit a 1 GiB budget and fails with NQ_ENOMEM,
    while the small requests around it are served."""
    big = nqueens.engine.job_device_bytes(nqueens.CountJob(22), 152)
    assert big > 4 << 30
    jobs = [nqueens.CountJob(8), nqueens.CountJob(22), nqueens.CountJob(10)]
    with srv_mod.Server(engine=FakeEngine(real_sizing=True), poll_us=100, budget_bytes=1 << 30) as s:
        futs = [s.submit(j) for j in jobs]
        s.drain(60)
        assert futs[0].result() == 92 and futs[2].result() == 724
        with pytest.raises(NQError) as e:
            futs[1].result()
        assert e.value.status == -5
    assert all(not any(j.N == 22 for j in b.jobs) for b in fake.created)   # never built


def test_real_sizes_cover_every_board():
    """The sizing call covers every board (the old fixed table stopped at N=21): its upper estimate holds
    each task's record, root, info and schedule plus the split queue, so it grows with N at a fixed split
    depth, and a forced split depth raises it."""
    by_n = {n: nqueens.engine.job_device_bytes(nqueens.CountJob(n), 152) for n in (10, 17, 19, 20, 21, 22)}
    assert by_n[17] < by_n[19] < by_n[20] < by_n[21] < by_n[22]
    assert by_n[10] < by_n[17]
    assert by_n[19] > 897071 * (16 + 16 + 8)            # N=19: records + roots + info at least
    assert nqueens.engine.job_device_bytes(nqueens.CountJob(19), 152, 2) > by_n[19]
    c = nqueens.engine.job_device_bytes(nqueens.CompletionJob(18, [(0, 3), (5, 7)]), 152)
    assert 0 < c < by_n[19]


def test_timing_table_recalibrates_from_measured_batches(fake):
    fake.delay_s = 0.05
    with srv_mod.Server(engine=FakeEngine(), poll_us=100) as s:
        assert s._count_ms[16] == srv_mod._COUNT_MS[16]
        s.submit(nqueens.CountJob(16)).result(timeout=30)
        s.drain(30)
        assert s._count_ms[16] > 10 * srv_mod._COUNT_MS[16]   # the fake's 50 ms run replaced the GB300 entry
