#!/usr/bin/env python3
"""Benchmark of the constellation DFS hot path on GB300 (one JSON line).

Workload: the plain single-N count at N=19 -- all 897,071 tasks of the
reference's preset-6 constellation set (4,968,057,848 solutions) -- one launch
sequence (prepare + DFS) per step.  metric = DFS nodes/s, where a node is one
candidate-queen extraction of the reference's dfs_iter
(14Bit_codon_GPU/356Py_savesp_narrow.py:1904-1965) and the per-N node totals
are frozen constants counted once by the CPU oracle (DFS_NODES below).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value: inputs resident in HBM, device-timed (CUDA events on the launching
stream), L2 flushed (256 MiB write) between timed steps.  e2e: the same
metric through the C ABI call nq_exec_solutions with pinned host records,
host->device copy and device->host read-back inside the timed region.
batch / serve: the metric's second half (the 256-job mixed batch and the
served completion stream, each against one plain launch per job).
--impl reference: the reference algorithm's CPU implementation on the host
cores (the C oracle port, all threads) on the same workload: the full task
list cut into one strided slice per timed step.  Multi-GPU: one process per GPU (torchrun), each rank counts the
full N=19 workload (replicas, weak scaling); value = all ranks' nodes / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(REPO, "n-queens_gb300"), os.path.join(REPO, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

# DFS nodes per N at the reference's dynamic preset (select_dynamic_preset_queens), counted by
# oracle.exec_solutions(N, oracle.gen_constellations(N, preset), want_nodes=True).
DFS_NODES = {10: 4980, 11: 27032, 12: 145880, 13: 787610, 14: 4578224, 15: 27864613, 16: 182533515,
             17: 1247485360, 18: 9087554384, 19: 69276398858, 20: 557537122738, 21: 4670180074483}
N_BENCH = 19          # the headline workload; --n selects another board (tests use small ones)
OPS_PER_NODE = 12   # INT32 ops per node in the reference hot loop (neg, and, xor, or, shl, or, shr, or, or, or, andnot, cmp)


def metric(N: int) -> str:
    return f"N={N} DFS nodes/s"


def preset_of(N: int) -> int:
    import oracle
    return oracle.preset_for(N)


def expected_total(N: int) -> int:
    import oracle
    return oracle.EXPECTED_TOTAL[N]


def load_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return json.load(f)
    except OSError:
        return None


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        # raw samples; NQ_CLOCKS_DIR keeps them somewhere chosen (default: the temp directory)
        import tempfile
        d = os.environ.get("NQ_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(d, f"clocks_bench_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sms)}


_ORACLE_RECORDS = {}


def oracle_records(N: int, preset: int):
    """The reference's task list for (N, preset), made by the oracle's own generator (no engine code)."""
    import oracle
    oracle.build()
    if (N, preset) not in _ORACLE_RECORDS:
        _ORACLE_RECORDS[(N, preset)] = oracle.gen_constellations(N, preset)
    return _ORACLE_RECORDS[(N, preset)]


def take(rec, idx):
    import oracle
    return oracle.Records(rec.ld[idx], rec.rd[idx], rec.col[idx], rec.startijkl[idx])


def cpu_sample(N: int, frac: float, seed: int):
    """Seeded subset of the N-workload's records (oracle generator) for the CPU legs."""
    import numpy as np
    recs = oracle_records(N, preset_of(N))
    rng = np.random.default_rng(seed)
    n = max(1, int(round(frac * len(recs))))
    idx = np.sort(rng.choice(len(recs), size=n, replace=False))
    return take(recs, idx), len(recs)


def run_cpu(N: int, target_s: float, seed: int = 2026):
    """Oracle port on all host threads over a sample sized to ~target_s seconds; returns nodes/s etc."""
    import oracle
    threads = os.cpu_count() or 1
    # calibrate on a small slice, then size the sample
    rec, m_all = cpu_sample(N, 1 / 512, seed)
    t0 = time.perf_counter()
    _, nodes = oracle.exec_solutions(N, rec, threads=threads, want_nodes=True)
    dt = max(time.perf_counter() - t0, 1e-3)
    rate = float(nodes.sum()) / dt
    frac = min(1.0, max(1 / 512, target_s * rate / DFS_NODES[N]))
    rec, m_all = cpu_sample(N, frac, seed + 1)
    t0 = time.perf_counter()
    _, nodes = oracle.exec_solutions(N, rec, threads=threads, want_nodes=True)
    dt = time.perf_counter() - t0
    n = int(nodes.sum())
    return {"value": n / dt, "nodes": n, "seconds": dt, "cores": threads, "tasks": len(rec), "tasks_all": m_all,
            "frac": frac}


def bench_config(N: int):
    """The workload both arms measure (the same dict on both lines)."""
    p = preset_of(N)
    m = len(oracle_records(N, p))
    return {"workload": f"plain single-N count, N={N}, preset {p} ({m:,} tasks, {expected_total(N):,} solutions)",
            "N": N, "preset": p, "tasks": m, "l2": "GPU arm: flushed between timed steps (256 MiB write)"}


def reference_arm(args):
    """The reference algorithm's CPU implementation (the oracle port of 356Py's generator and dfs_iter) on all
    host threads.  The full N=19 task list is cut into `steps` strided slices; timed step i counts slice i, so
    the timed steps together count every task once and the total must equal the known answer."""
    import numpy as np
    import oracle
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    N = args.n
    rec = oracle_records(N, preset_of(N))
    m = len(rec)
    rng = np.random.default_rng(2026)
    for _ in range(args.warmup):                       # warm-up: small seeded samples, untimed
        oracle.exec_solutions(N, take(rec, np.sort(rng.choice(m, size=max(1, m // 512), replace=False))),
                              threads=threads)
    K = max(1, args.steps)
    secs, nodes_total, sol_total = [], 0, 0
    for i in range(K):
        sub = take(rec, np.arange(i, m, K))
        t0 = time.perf_counter()
        sol, nodes = oracle.exec_solutions(N, sub, threads=threads, want_nodes=True)
        secs.append(time.perf_counter() - t0)
        nodes_total += int(nodes.sum())
        sol_total += int(sol.sum())
    assert sol_total == expected_total(N), f"reference arm total {sol_total} != {expected_total(N)}"
    assert nodes_total == DFS_NODES[N]
    v = nodes_total / sum(secs)
    sample = (f"the full N={N} preset-{preset_of(N)} task list ({m} tasks, oracle generator) cut into {K} strided "
              "slices, one per "
              f"timed step; the steps together count every task once (total {sol_total}); nodes from the oracle's "
              "own dfs_iter counter")
    line = {
        "impl": "reference", "metric": metric(N), "value": v, "unit": "nodes/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": bench_config(N),
        "cpu_baseline": {"value": v, "unit": "nodes/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "nodes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "total": sol_total, "seconds_total": sum(secs),
        "note": ("CPU implementation of the reference algorithm (C restatement of 356Py gen_constellations and "
                 "dfs_iter, oracle/nq_oracle.c, pthreads); the reference's own C port "
                 "(10Bit_CUDA/13CUDA_constellation.c) is built from the reference checkout, which the GPU host does "
                 "not have"),
    }
    print(json.dumps(line))
    return 0


def read_profile_figure(key):
    """A per-launch figure of the dfs_kernel N=19 ncu capture (profiles/dfs_kernel_n19_traffic.txt), or None."""
    p = os.path.join(REPO, "profiles", "dfs_kernel_n19_traffic.txt")
    try:
        for line in open(p):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def read_traffic():
    """dram bytes per dfs_kernel launch from the committed ncu summary, or None."""
    return read_profile_figure("dram_bytes_per_launch")


def ours_arm(args):
    import numpy as np
    import torch
    import nqueens

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    eng = nqueens.Engine(dev, block=args.block, split=args.split)
    N = args.n
    expected = expected_total(N)
    recs = nqueens.gen_records(N)
    m = len(recs)
    start_min = int((recs["startijkl"] >> 20).min())
    d_rec = torch.from_numpy(recs.view(np.uint8).copy()).to(f"cuda:{dev}")
    d_total = torch.zeros(1, dtype=torch.int64, device=f"cuda:{dev}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
    s = torch.cuda.Stream(device=dev)

    def step():
        eng.exec_device(N, d_rec.data_ptr(), m, start_min, d_total.data_ptr(), 0, s.cuda_stream)

    for _ in range(args.warmup):
        step()
        eng.sync()
        assert int(d_total.item()) == expected, f"N={N} total mismatch"
    peaks = load_peaks()
    int_peak = eng.int32_peak(0)
    int_peak_add = eng.int32_peak(1)

    clocks = Clocks(dev)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    dfs_ms = []
    for i in range(args.steps):
        with torch.cuda.stream(s):
            flush.zero_()                      # L2 flush (256 MiB > 129 MB L2), outside the timed events
            ev[i][0].record(s)
        step()
        with torch.cuda.stream(s):
            ev[i][1].record(s)
        eng.sync()
        dfs_ms.append(eng.last_kernel_ms()[1])
        assert int(d_total.item()) == expected
    split_depth, queued = eng.last_run_info()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_ms = sum(step_ms)
    if ws > 1:
        t = torch.tensor([t_ms], device=f"cuda:{dev}", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_ms = float(t.item())
    ms_per_step = t_ms / args.steps
    nodes = DFS_NODES[N]
    value = ws * nodes * args.steps / (t_ms * 1e-3)

    # e2e: host records (pinned) -> C ABI -> host total
    pinned = torch.empty(m * 16, dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = recs.view(np.uint8)
    h_recs = pinned.numpy().view(nqueens.RECORD_DTYPE)
    e2e_t = []
    for i in range(args.steps + 1):
        flush.zero_(); torch.cuda.synchronize()
        t0 = time.perf_counter()
        tot, _ = eng.exec_records(N, h_recs)
        e2e_t.append(time.perf_counter() - t0)
        assert tot == expected
    e2e_s = statistics.mean(e2e_t[1:])
    # the reference's "wall s per N": generation + upload + count + read-back through nq_count
    t0 = time.perf_counter()
    assert eng.count(N).total == expected
    wall_s = time.perf_counter() - t0

    dfs_avg = statistics.mean(dfs_ms)
    achieved_ops = nodes * OPS_PER_NODE / (dfs_avg * 1e-3)
    at_profile = N == 19                     # the committed ncu capture is of the N=19 launch
    traffic = read_traffic() if at_profile else None
    # Executed instructions against the issue limit (one warp instruction per clock per SM sub-partition):
    # the step is issue/math-pipe bound, so this is the fraction that measures the kernel.
    warp_instr = read_profile_figure("warp_instructions_per_launch") if at_profile else None
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    issue = None
    if warp_instr and clk.get("sm_mhz"):
        peak_wi = sm_count * 4 * clk["sm_mhz"] * 1e6
        got_wi = warp_instr / (dfs_avg * 1e-3)
        issue = {"warp_instructions_per_launch": warp_instr, "achieved": got_wi / 1e9, "peak": peak_wi / 1e9,
                 "unit": "G warp-instr/s", "frac": got_wi / peak_wi,
                 "source": "instruction count of one ncu capture (profiles/dfs_kernel_n19.md), time of this run, "
                           "peak = SMs x 4 issue slots x median sampled SM clock"}
    line = {
        "metric": metric(N), "value": value, "unit": "nodes/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": bench_config(N),
        "launch": {"per_step": "one prepare + split + DFS launch sequence", "block": eng.get_config()[0],
                   "split_depth": split_depth, "queued_subtasks": queued, "parallelism": f"replicas x{ws}"},
        "total": expected,
        "wall_s": wall_s,
        "dfs_kernel_ms": dfs_avg,
        "e2e": {"value": ws * nodes / e2e_s, "unit": "nodes/s", "seconds_per_step": e2e_s,
                "h2d_bytes_per_step": m * 16, "d2h_bytes_per_step": 16},
        "roofline": {"bound": "alu", "achieved": achieved_ops / 1e9, "peak": int_peak / 1e9, "unit": "Gop/s",
                     "frac": achieved_ops / int_peak, "traffic": traffic,
                     "peak_source": "measured in this run: lop3.b32 throughput probe (nq_int32_peak); "
                                    f"add.u32 probe {int_peak_add / 1e9:.0f} Gop/s",
                     "ops_per_node": OPS_PER_NODE, "issue": issue,
                     "alu_pipe_pct_of_peak_ncu": read_profile_figure("alu_pipe_pct_of_peak") if at_profile else None,
                     "issue_active_pct_ncu": read_profile_figure("issue_active_pct") if at_profile else None,
                     "hbm_frac": (m * 16 + m * 16 + m * 8 + m * 4 * 15) / (dfs_avg * 1e-3) / (
                         (peaks or {}).get("hbm_gbs", 6800.0) * 1e9)},
        "clocks": clk,
        "gpu_launches": (4 if split_depth > 0 else 2) * args.steps,
    }
    if rank == 0 and not args.no_cpu:
        cb = run_cpu(N, args.cpu_seconds)
        line["cpu_baseline"] = {"value": cb["value"], "unit": "nodes/s", "cores": cb["cores"], "kind": "port",
                                "sample": (f"seeded {cb['frac']:.4f} of the N={N} task list ({cb['tasks']} tasks, "
                                           f"oracle generator, {cb['seconds']:.1f} s), C oracle port, all host "
                                           "threads")}
    # the metric's second half: the mixed batch and the served stream against one plain launch per job
    if rank == 0 and not args.no_mix:
        line["batch"] = batch_figures(eng, max(3, min(args.steps, 5)), value / ws)
        line["serve"] = serve_figures(eng, args)
    if rank == 0:
        print(json.dumps(line))
    eng.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def dfs_ms_alone(eng, N: int, reps: int = 3) -> float:
    """Device time of N's whole-board DFS launch run alone (records resident, the engine's tuned launch)."""
    import numpy as np
    import torch
    import nqueens
    recs = nqueens.gen_records(N)
    start_min = int((recs["startijkl"] >> 20).min())
    d_rec = torch.from_numpy(recs.view(np.uint8).copy()).cuda()
    d_total = torch.zeros(1, dtype=torch.int64, device="cuda")
    eng._apply_tuning(N)
    ts = []
    for r in range(reps + 1):
        eng.exec_device(N, d_rec.data_ptr(), len(recs), start_min, d_total.data_ptr())
        eng.sync()
        if r:
            ts.append(eng.last_kernel_ms()[1])
    return statistics.median(ts)


def batch_figures(eng, reps: int, node_rate: float = 0.0) -> dict:
    """256 counting jobs, N uniform in 10..18 (numpy default_rng(2026)), tasks resident: one graph-replayed
    persistent launch against one launch and read-back per job, and the floor both forms share (the sum of each
    job's DFS kernel time when it runs alone)."""
    import numpy as np
    import nqueens
    import oracle
    Ns = [int(x) for x in np.random.default_rng(2026).integers(10, 19, size=256)]
    exp = np.array([oracle.EXPECTED_TOTAL[N] for N in Ns], np.uint64)
    t0 = time.perf_counter()
    b = eng.batch([nqueens.CountJob(N) for N in Ns])
    build_s = time.perf_counter() - t0
    try:
        for _ in range(2):
            assert np.array_equal(b.run(use_graph=True), exp) and np.array_equal(b.run_plain(), exp)
        tg, tp = [], []
        for _ in range(reps):
            t0 = time.perf_counter(); r = b.run(use_graph=True); tg.append(time.perf_counter() - t0)
            assert np.array_equal(r, exp)
            t0 = time.perf_counter(); r = b.run_plain(); tp.append(time.perf_counter() - t0)
            assert np.array_equal(r, exp)
        tasks, h2d = b.tasks, b.h2d_bytes
    finally:
        b.close()
    alone = {N: dfs_ms_alone(eng, N) for N in sorted(set(Ns))}
    floor_ms = sum(alone[N] for N in Ns)
    # the work floor: every job's reference nodes at the full-GPU node rate of the N=19 count (no mix can beat it
    # by more than the few percent the kernel's pruning varies between boards)
    work_ms = 1e3 * sum(DFS_NODES[N] for N in Ns) / node_rate if node_rate > 0 else None
    g, p = statistics.median(tg), statistics.median(tp)
    return {"workload": "256 counting jobs, N uniform 10..18 (numpy default_rng(2026)), tasks resident",
            "jobs": len(Ns), "tasks": tasks, "jobs_per_s": len(Ns) / g, "ms": 1e3 * g,
            "plain_jobs_per_s": len(Ns) / p, "plain_ms": 1e3 * p, "speedup_vs_plain": p / g,
            "floor_ms": floor_ms, "ms_over_floor": 1e3 * g / floor_ms,
            "floor": "sum over the 256 jobs of the job's whole-board DFS kernel time alone (CUDA events)",
            "work_floor_ms": work_ms,
            "work_floor": "sum over the 256 jobs of the job's reference DFS nodes / this run's N=19 nodes per second",
            "dfs_ms_alone_by_N": {str(k): round(v, 4) for k, v in alone.items()},
            "build_s": build_s, "h2d_bytes": h2d, "exact": True, "reps": reps}


def serve_figures(eng, args) -> dict:
    """The served completion stream (N uniform 14..20, k uniform 0..4 pre-placed queens, seeded) offered all at
    once, so jobs/s is each form's capacity: the continuous-batching server against one plain call per query in
    arrival order.  Latency = result time - submission time; counts must agree query for query."""
    import numpy as np
    import nqueens
    from nqueens.server import Server, random_completion_queries, run_plain
    jobs = random_completion_queries(args.queries, seed=2026, N_range=(14, 20), k_range=(0, 4))
    run_plain(eng, jobs[:4])                           # warm-up
    for j in jobs:                                     # whole-board sizes are cached per board: size them once
        if isinstance(j, nqueens.CountJob):
            eng.job_device_bytes(j)
    t0 = time.perf_counter()
    lat_plain, res_plain = [], []
    for j in jobs:
        res_plain.append(run_plain(eng, [j])[0])
        lat_plain.append(time.perf_counter() - t0)
    span_plain = time.perf_counter() - t0
    with Server(engine=eng, budget_bytes=args.budget_gb << 30, max_inflight=args.inflight,
                max_batch_jobs=args.max_batch, large_share=args.large_share) as srv:
        futs = [srv.submit(j) for j in jobs]
        srv.drain(600)
        res_srv = [f.result() for f in futs]
        st = srv.stats()
    assert res_srv == res_plain, "served counts differ from the plain per-query counts"
    pl = np.array(lat_plain)
    return {"workload": f"{len(jobs)} completion queries (numpy default_rng(2026)), all offered at t=0",
            "queries": len(jobs), "jobs_per_s": st.jobs_per_s, "p50_ms": 1e3 * st.percentile(50),
            "p99_ms": 1e3 * st.percentile(99), "batches": st.batches,
            "plain": {"jobs_per_s": len(jobs) / span_plain, "p50_ms": 1e3 * float(np.percentile(pl, 50)),
                      "p99_ms": 1e3 * float(np.percentile(pl, 99))},
            "speedup_vs_plain": st.jobs_per_s * span_plain / len(jobs),
            "h2d_bytes": st.h2d_bytes, "d2h_bytes": st.d2h_bytes, "exact": True}


def batch_arm(args):
    """Config: 256 counting jobs, N uniform in 10..18 from numpy default_rng(2026), tasks resident,
    all in one graph-captured persistent launch vs one launch and read-back per job."""
    import numpy as np
    import torch
    import nqueens
    rng = np.random.default_rng(2026)
    Ns = [int(x) for x in rng.integers(10, 19, size=256)]
    eng = nqueens.Engine(0, block=args.block)
    want = [eng.count(N).total for N in sorted(set(Ns))]
    want = dict(zip(sorted(set(Ns)), want))
    t0 = time.perf_counter()
    b = eng.batch([nqueens.CountJob(N) for N in Ns])
    build_s = time.perf_counter() - t0
    exp = np.array([want[N] for N in Ns], np.uint64)
    for _ in range(args.warmup):
        assert np.array_equal(b.run(use_graph=True), exp)
        assert np.array_equal(b.run_plain(), exp)
    t_graph, t_plain = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter(); r = b.run(use_graph=True); t_graph.append(time.perf_counter() - t0)
        assert np.array_equal(r, exp)
        t0 = time.perf_counter(); r = b.run_plain(); t_plain.append(time.perf_counter() - t0)
        assert np.array_equal(r, exp)
    # drop-in per job: nq_count (host generation, upload, prepare, split, DFS, read-back) for every job
    t0 = time.perf_counter()
    for N in Ns:
        assert eng.count(N).total == want[N]
    dropin_s = time.perf_counter() - t0
    g, p = statistics.mean(t_graph), statistics.mean(t_plain)
    # where batching pays: a mix of small boards (N uniform 6..14), launch-bound in the plain form
    small_Ns = [int(x) for x in np.random.default_rng(2026).integers(6, 15, size=256)]
    sb = eng.batch([nqueens.CountJob(N) for N in small_Ns])
    sexp = np.array([eng.count(N).total for N in small_Ns], np.uint64)
    assert np.array_equal(sb.run(use_graph=True), sexp) and np.array_equal(sb.run_plain(), sexp)
    sg, sp = [], []
    for _ in range(max(3, args.steps)):
        t0 = time.perf_counter(); sb.run(use_graph=True); sg.append(time.perf_counter() - t0)
        t0 = time.perf_counter(); sb.run_plain(); sp.append(time.perf_counter() - t0)
    sb.close()
    small = {"jobs": 256, "N": "uniform 6..14", "graph_jobs_per_s": 256 / statistics.mean(sg),
             "plain_resident_jobs_per_s": 256 / statistics.mean(sp),
             "speedup_vs_plain_resident": statistics.mean(sp) / statistics.mean(sg)}
    line = {"metric": "mixed-batch jobs/s (256 jobs, N~U{10..18})", "value": len(Ns) / g, "unit": "jobs/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * g, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": "256 counting jobs, N uniform 10..18 (numpy default_rng(2026)), one graph-captured "
                                   "persistent launch per step, tasks resident", "jobs": len(Ns),
                       "tasks": b.tasks, "block": args.block},
            "plain_resident_jobs_per_s": len(Ns) / p, "plain_resident_ms": 1e3 * p,
            "speedup_vs_plain_resident": p / g,
            "batch_build_s": build_s, "e2e": {"value": len(Ns) / (build_s + g), "unit": "jobs/s",
                                              "seconds_per_step": build_s + g,
                                              "h2d_bytes_per_step": b.h2d_bytes, "d2h_bytes_per_step": 8 * len(Ns)},
            "plain_dropin_jobs_per_s": len(Ns) / dropin_s, "speedup_e2e_vs_dropin": dropin_s / (build_s + g),
            "small_mix": small, "gpu_launches": 1}
    b.close()
    eng.close()
    print(json.dumps(line))
    return 0


def serve_arm(args):
    """Config: served completion stream -- N uniform 14..20, k uniform 0..4 pre-placed queens (seeded),
    Poisson arrivals at a stated rate, admission by device-memory budget; vs the plain per-query launch."""
    import numpy as np
    import nqueens
    from nqueens.server import Server, random_completion_queries, run_plain
    jobs = random_completion_queries(args.queries, seed=2026, N_range=(14, 20), k_range=(0, 4))
    rng = np.random.default_rng(7)
    gaps = rng.exponential(1.0 / args.rate, size=len(jobs))
    eng = nqueens.Engine(0, block=args.block)
    run_plain(eng, jobs[:4])                         # warm-up (module load, allocations)
    for j in jobs:                                   # whole-board sizes are cached per board: size them once
        if isinstance(j, nqueens.CountJob):
            eng.job_device_bytes(j)
    # plain: one query at a time, FIFO, same arrival times
    arrivals = np.cumsum(gaps)
    t_start = time.perf_counter()
    lat_plain, res_plain = [], []
    for j, a in zip(jobs, arrivals):
        now = time.perf_counter() - t_start
        if now < a:
            time.sleep(a - now)
        r = run_plain(eng, [j])[0]
        res_plain.append(r)
        lat_plain.append(time.perf_counter() - t_start - a)
    span_plain = time.perf_counter() - t_start
    with Server(engine=eng, budget_bytes=args.budget_gb << 30, max_inflight=args.inflight,
                max_batch_jobs=args.max_batch, large_share=args.large_share) as srv:
        t_start = time.perf_counter()
        futs = []
        for j, a in zip(jobs, arrivals):
            now = time.perf_counter() - t_start
            if now < a:
                time.sleep(a - now)
            futs.append(srv.submit(j))
        srv.drain(600)
        res_srv = [f.result() for f in futs]
        st = srv.stats()
    assert res_srv == res_plain, "served counts differ from the plain per-query counts"
    lat_srv = [f_lat for f_lat in st.latencies_by_request] if hasattr(st, "latencies_by_request") else None
    if lat_srv is not None:
        worst = sorted(range(len(jobs)), key=lambda i: -lat_srv[i])[:6]
        for i in worst:
            j = jobs[i]
            q, b, r = st.phases_by_request[i]
            print(f"serve tail: job {i} N={j.N} k={len(getattr(j, 'queens', []))} arrival={arrivals[i]:.2f}s "
                  f"served={1e3 * lat_srv[i]:.0f}ms (queued {1e3 * q:.0f}, build {1e3 * b:.0f}, run {1e3 * r:.0f}) "
                  f"plain={1e3 * lat_plain[i]:.0f}ms", file=sys.stderr)
    eng.close()
    pl = np.array(lat_plain)
    line = {"metric": "served completion stream jobs/s (N~U{14..20}, k~U{0..4})", "value": st.jobs_per_s,
            "unit": "jobs/s", "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": 1e3 * st.makespan_s,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": f"{len(jobs)} queries, Poisson arrivals {args.rate}/s (numpy default_rng(2026) "
                                   "boards, default_rng(7) gaps), continuous batching",
                       "budget_gb": args.budget_gb, "max_inflight": args.inflight, "max_batch_jobs": args.max_batch,
                       "large_share": args.large_share},
            "p50_ms": 1e3 * st.percentile(50), "p90_ms": 1e3 * st.percentile(90), "p99_ms": 1e3 * st.percentile(99),
            "max_ms": 1e3 * max(st.latencies_s), "batches": st.batches,
            "max_inflight_seen": st.max_inflight_seen,
            "plain": {"jobs_per_s": len(jobs) / span_plain, "p50_ms": 1e3 * float(np.percentile(pl, 50)),
                      "p90_ms": 1e3 * float(np.percentile(pl, 90)), "p99_ms": 1e3 * float(np.percentile(pl, 99)),
                      "max_ms": 1e3 * float(pl.max())},
            "e2e": {"value": st.jobs_per_s, "unit": "jobs/s", "h2d_bytes_per_step": st.h2d_bytes,
                    "d2h_bytes_per_step": st.d2h_bytes},
            "exact": True}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--n", type=int, default=N_BENCH, choices=sorted(DFS_NODES), help="board size of the workload")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--block", type=int, default=64,
                    help="threads per block; 64 with --split -1 keeps the autotuned per-N table (nqueens/tuning.json)")
    ap.add_argument("--split", type=int, default=-1, help="split depth (-1 automatic)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mix", action="store_true", help="skip the batch and serve figures of the default line")
    ap.add_argument("--workload", choices=["n19", "batch", "serve"], default="n19",
                    help="n19: the headline single-N count; batch / serve: the batching and serving configs")
    ap.add_argument("--queries", type=int, default=150)
    ap.add_argument("--rate", type=float, default=10.0, help="serve: Poisson arrival rate (queries/s)")
    ap.add_argument("--budget-gb", type=int, default=32)
    ap.add_argument("--inflight", type=int, default=3)
    ap.add_argument("--max-batch", type=int, default=16)
    ap.add_argument("--large-share", type=float, default=0.875,
                    help="serve: share of the resident DFS blocks given to the large-request lane")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "batch":
        return batch_arm(args)
    if args.workload == "serve":
        return serve_arm(args)
    return ours_arm(args)


if __name__ == "__main__":
    sys.exit(main())
