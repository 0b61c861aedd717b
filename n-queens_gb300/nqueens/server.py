"""Continuous-batching request loop (no reference counterpart: the reference
counts one N per process run).

Requests -- whole-board counts (``CountJob``) and completion queries with
pre-placed queens (``CompletionJob``) -- are queued as they arrive and sorted
into two lanes by their estimated GPU time.  Large requests (a whole N=20
board, say) each get a batch of their own whose persistent kernel holds most
of the resident blocks; small requests that arrive meanwhile are gathered
into batches on the remaining share of the GPU, so they never queue behind a
large one.  A scheduler thread admits a lane's queued requests as a new
batch whenever that lane has a free slot and the device-memory budget allows:
the batch's tasks are built and uploaded (``nq_batch_create``), then launched
asynchronously on the batch's own CUDA stream (``nq_batch_submit``), so
batches admitted while others run overlap them on the GPU.  Each request is
sized when it is submitted (``nq_job_device_bytes``, host-side, no allocation),
so the budget is a hard limit: a request larger than the whole budget fails
at once with NQ_ENOMEM, and the bytes in flight never exceed it.  Finished batches
are polled (bounded waits), their per-job totals resolve the requests'
futures, and their device memory returns to the budget.

Counts are exact integers: a request's result is the same alone and in any
mix (tests/test_server.py checks it).  Each request records its latency
(arrival to result); ``stats()`` reports p50/p99 and jobs/s.
"""
from __future__ import annotations

import collections
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Deque, List, Optional, Sequence

import numpy as np

from ._lib import NQError
from .engine import Batch, CompletionJob, CountJob, Engine


@dataclass
class _Request:
    job: object
    future: Future
    t_arrival: float
    seq: int = 0
    t_admit: float = 0.0    # taken off the queue into a batch
    t_built: float = 0.0    # its batch built and launched
    t_done: float = 0.0
    bytes: int = 0          # device bytes of the request, sized when it was submitted


@dataclass
class _InFlight:
    batch: Batch
    requests: List[_Request]
    bytes: int
    large: bool = False


# GPU milliseconds of a whole-board count, the starting point of each server's table: measured on
# GB300 with bench-style timing; a server replaces an entry with the run time it measures for a
# single-request batch of that board (exponential average), so another GPU recalibrates itself.
_COUNT_MS = {16: 0.5, 17: 2.2, 18: 13.0, 19: 86.0, 20: 670.0, 21: 5600.0}


def estimate_ms(job, table: Optional[dict] = None) -> float:
    """Rough GPU time of a request: a whole board from the table; k pre-placed queens cut the
    unweighted search (8x the symmetric one) by about N per queen."""
    N = job.N
    t = _COUNT_MS if table is None else table
    base = t.get(N)
    if base is None:   # outside the table: about 9x per board size from its nearest entry
        near = min(t, key=lambda n: abs(n - N))
        base = t[near] * 9.0 ** (N - near)
    if isinstance(job, CountJob):
        return base
    k = len(job.queens)
    if k == 0:
        return base * 8.0
    return base * 8.0 / float(N) ** k


@dataclass
class ServerStats:
    completed: int
    latencies_s: List[float] = field(default_factory=list)
    latencies_by_request: List[float] = field(default_factory=list)   # in submission order
    phases_by_request: List[tuple] = field(default_factory=list)      # (queued, build, run) seconds
    h2d_bytes: int = 0              # copied to the device by every batch's build
    d2h_bytes: int = 0              # per-job totals read back
    makespan_s: float = 0.0
    batches: int = 0
    max_inflight_seen: int = 0
    max_admitted_bytes: int = 0     # largest sum of the sized requests in flight at once

    def percentile(self, q: float) -> float:
        return float(np.percentile(self.latencies_s, q)) if self.latencies_s else 0.0

    @property
    def jobs_per_s(self) -> float:
        return self.completed / self.makespan_s if self.makespan_s > 0 else 0.0


class Server:
    """Admit requests into batches by device-memory budget and keep several batches in flight."""

    def __init__(self, device: int = 0, budget_bytes: int = 16 << 30, max_inflight: int = 3,
                 max_batch_jobs: int = 64, use_graph: bool = False, engine: Optional[Engine] = None,
                 poll_us: int = 200, share_gpu: bool = True, large_ms: float = 50.0, large_share: float = 0.875):
        self.engine = engine or Engine(device)
        # Lanes: requests estimated above large_ms run one per batch on large_share of the
        # resident blocks; the rest are batched on the remaining share while a large batch
        # runs (share_gpu), so a small request admitted then starts at once beside it, and on
        # the whole GPU otherwise.  Shares are taken of each batch's own resident capacity
        # (its stack depth sets how many blocks fit on an SM).
        self.share_gpu = bool(share_gpu)
        self.large_share = float(large_share)
        self.large_ms = float(large_ms)
        self.budget = int(budget_bytes)
        self.max_inflight = int(max_inflight)
        self.max_batch_jobs = int(max_batch_jobs)
        self.use_graph = use_graph
        self.poll_us = int(poll_us)
        self._pending: Deque[_Request] = collections.deque()        # small requests
        self._pending_large: Deque[_Request] = collections.deque()  # large requests
        self._inflight: List[_InFlight] = []
        self._building = 0
        self._seq = 0
        self._h2d = 0
        self._admitted = 0
        self._cv = threading.Condition()
        self._stop = False
        self._done: List[_Request] = []
        self._batches = 0
        self._max_inflight_seen = 0
        self._max_admitted = 0
        self._t0: Optional[float] = None
        self._t_last = 0.0
        self._error: Optional[BaseException] = None
        self._count_ms = dict(_COUNT_MS)   # recalibrated from measured single-board batches
        self._thread = threading.Thread(target=self._loop, name="nqueens-server", daemon=True)
        self._thread.start()

    # -- client side ---------------------------------------------------------
    def submit(self, job) -> Future:
        if not isinstance(job, (CountJob, CompletionJob)):
            raise TypeError("submit a CountJob or a CompletionJob")
        f: Future = Future()
        now = time.perf_counter()
        # Size the request here, on the caller's thread and outside the server's lock: the first sizing of a
        # large board generates its constellations (about a second at N=22), which must not stall the scheduler.
        try:
            nbytes = self._job_bytes(job)
        except NQError as exc:
            f.set_exception(exc)
            return f
        if nbytes > self.budget:               # can never fit: fails alone, nothing is queued
            f.set_exception(NQError(-5, f"request needs about {nbytes} device bytes, more than the server's "
                                        f"budget of {self.budget}"))
            return f
        with self._cv:
            if self._error is not None:
                raise RuntimeError("server stopped after an error") from self._error
            if self._t0 is None:
                self._t0 = now
            r = _Request(job, f, now, self._seq, bytes=nbytes)
            self._seq += 1
            (self._pending_large if estimate_ms(job, self._count_ms) > self.large_ms else self._pending).append(r)
            self._cv.notify()
        return f

    def drain(self, timeout_s: float = 600.0) -> None:
        """Wait until every submitted request has a result (bounded)."""
        t_end = time.perf_counter() + timeout_s
        with self._cv:
            while self._pending or self._pending_large or self._inflight or self._building:
                if self._error is not None:
                    raise RuntimeError("server failed") from self._error
                left = t_end - time.perf_counter()
                if left <= 0:
                    raise TimeoutError("requests still running after the drain timeout")
                self._cv.wait(min(left, 0.05))

    def stats(self) -> ServerStats:
        with self._cv:
            lat = [r.t_done - r.t_arrival for r in self._done]
            done = sorted(self._done, key=lambda r: r.seq)
            by_req = [r.t_done - r.t_arrival for r in done]
            phases = [(r.t_admit - r.t_arrival, r.t_built - r.t_admit, r.t_done - r.t_built) for r in done]
            span = (self._t_last - self._t0) if self._t0 is not None else 0.0
            return ServerStats(completed=len(self._done), latencies_s=lat, latencies_by_request=by_req,
                               phases_by_request=phases, h2d_bytes=self._h2d, d2h_bytes=8 * len(self._done),
                               makespan_s=span, batches=self._batches, max_inflight_seen=self._max_inflight_seen,
                               max_admitted_bytes=self._max_admitted)

    def close(self) -> None:
        with self._cv:
            self._stop = True
            self._cv.notify()
        self._thread.join(timeout=60)
        for f in self._inflight:
            f.batch.close()
        self._inflight.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- scheduler thread ------------------------------------------------------
    def _collect(self) -> bool:
        progressed = False
        for fl in list(self._inflight):
            out = fl.batch.poll(0)
            if out is None:
                continue
            now = time.perf_counter()
            for r, v in zip(fl.requests, out.tolist()):
                r.t_done = now
                r.future.set_result(int(v))
            if fl.requests:
                self._calibrate(fl, now - fl.requests[0].t_built)
            fl.batch.close()
            with self._cv:
                self._inflight.remove(fl)
                self._admitted -= fl.bytes
                self._done.extend(fl.requests)
                self._t_last = now
                self._cv.notify_all()
            progressed = True
        return progressed

    def _admit_lane(self, large: bool) -> bool:
        queue = self._pending_large if large else self._pending
        with self._cv:
            n_lane = sum(1 for f in self._inflight if f.large == large)
            slots = 1 if large else max(1, self.max_inflight - 1)
            if not queue or n_lane >= slots:
                return False
            take: List[_Request] = []
            est = 0
            while queue and len(take) < (1 if large else self.max_batch_jobs):
                e = queue[0].bytes
                if take and self._admitted + est + e > self.budget:
                    break
                if not take and self._admitted + e > self.budget:
                    return False          # wait for memory to free up
                take.append(queue.popleft())
                take[-1].t_admit = time.perf_counter()
                est += e
            if not take:
                return False
            self._building += 1          # taken off the queue, not yet in flight
        try:
            batch = Batch(self.engine, [r.job for r in take])   # host build + upload, other batches keep running
        except NQError as exc:
            self._reject(take, exc, queue)
            with self._cv:
                self._building -= 1
                self._cv.notify_all()
            return True
        # the sized estimate is an upper bound of the batch's bytes; count whichever is larger against the budget
        nbytes = max(est, int(batch.device_bytes))
        h2d = getattr(batch, "h2d_bytes", 0)
        if self.share_gpu:
            # small batches take the whole GPU while no large batch runs (they end in
            # milliseconds); beside a large batch they get the small lane's share
            with self._cv:
                large_running = any(f.large for f in self._inflight)
            share = self.large_share if large else (1.0 - self.large_share if large_running else 1.0)
            batch.set_grid(max(1, int(round(batch.resident_blocks() * share))))
        batch.submit(self.use_graph)
        t_built = time.perf_counter()
        for r in take:
            r.t_built = t_built
        with self._cv:
            self._inflight.append(_InFlight(batch, take, nbytes, large))
            self._h2d += h2d
            self._building -= 1
            self._admitted += nbytes
            self._max_admitted = max(self._max_admitted, self._admitted)
            self._batches += 1
            self._max_inflight_seen = max(self._max_inflight_seen, len(self._inflight))
        return True

    def _job_bytes(self, job) -> int:
        """Device bytes a request will take, from the engine's host-side sizing (nq_job_device_bytes)."""
        return int(self.engine.job_device_bytes(job))

    def _calibrate(self, fl: "_InFlight", seconds: float) -> None:
        """A batch holding one whole-board count measures that board's GPU time on this device."""
        if len(fl.requests) == 1 and isinstance(fl.requests[0].job, CountJob):
            N = fl.requests[0].job.N
            ms = 1e3 * seconds
            old = self._count_ms.get(N)
            self._count_ms[N] = ms if old is None else 0.5 * old + 0.5 * ms

    def _admit(self) -> bool:
        a = self._admit_lane(True)
        b = self._admit_lane(False)
        return a or b

    def _reject(self, take: List[_Request], exc: NQError, queue: Deque[_Request]) -> None:
        """A batch failed to build: build its requests one by one so only the bad ones fail."""
        for r in take:
            if len(take) > 1:
                try:
                    b = Batch(self.engine, [r.job])
                except NQError as e1:
                    r.future.set_exception(e1)
                    continue
                b.close()
                with self._cv:
                    queue.appendleft(r)              # valid: queue it again
            else:
                r.future.set_exception(exc)

    def _loop(self) -> None:
        try:
            while True:
                with self._cv:
                    idle = not self._pending and not self._pending_large and not self._inflight
                    if self._stop and idle:
                        return
                    if idle:
                        self._cv.wait(0.05)
                        continue
                progressed = self._collect()
                progressed = self._admit() or progressed
                if not progressed:
                    time.sleep(self.poll_us * 1e-6)
        except BaseException as exc:            # surface failures to the clients
            with self._cv:
                self._error = exc
                for r in list(self._pending) + list(self._pending_large):
                    r.future.set_exception(exc)
                self._pending.clear()
                self._pending_large.clear()
                for fl in self._inflight:
                    for r in fl.requests:
                        if not r.future.done():
                            r.future.set_exception(exc)
                self._cv.notify_all()


def random_completion_queries(n: int, seed: int, N_range=(14, 20), k_range=(0, 4)) -> List[object]:
    """The served completion stream of the workload: N uniform in N_range, k uniform
    in k_range pre-placed queens at seeded rows and columns, resampled while any two
    attack each other.  k == 0 is a whole-board count (CountJob)."""
    rng = np.random.default_rng(seed)
    out: List[object] = []
    for _ in range(n):
        N = int(rng.integers(N_range[0], N_range[1] + 1))
        k = int(rng.integers(k_range[0], k_range[1] + 1))
        if k == 0:
            out.append(CountJob(N))
            continue
        while True:
            rows = rng.choice(N, size=k, replace=False)
            cols = rng.integers(0, N, size=k)
            q = list(zip(rows.tolist(), cols.tolist()))
            if all(q[a][1] != q[b][1] and abs(q[a][0] - q[b][0]) != abs(q[a][1] - q[b][1])
                   for a in range(k) for b in range(a + 1, k)):
                break
        out.append(CompletionJob(N, q))
    return out


def run_plain(engine: Engine, jobs: Sequence) -> List[int]:
    """The plain form: one synchronous call (one launch sequence) per job, in order."""
    res = []
    for j in jobs:
        if isinstance(j, CountJob):
            res.append(engine.count(j.N, j.preset).total)
        else:
            res.append(engine.count_completions(j.N, j.queens))
    return res
