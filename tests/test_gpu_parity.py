"""GPU parity: the sm_103a kernels through the C ABI against the oracle and the
reference's golden vectors.  Bit-exact for every count."""
import json
import os

import numpy as np
import pytest

from conftest import REPO, gpu_available
from golden_util import canonical_order, solution_digest

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]
GOLDEN = os.path.join(REPO, "tests", "golden")


@pytest.fixture(scope="module")
def eng():
    import nqueens
    e = nqueens.Engine(0)
    yield e
    e.close()


def _o_records(oracle_mod, recs):
    return oracle_mod.Records(recs["ld"].astype(np.uint64), recs["rd"].astype(np.uint64),
                              recs["col"].astype(np.uint64), recs["startijkl"].copy())


@pytest.mark.parametrize("N", range(6, 20))
def test_per_record_counts_match_archived_solutions(eng, N):
    """Every record's weighted count equals the reference's archived solutions_N{N}_5_v2.bin."""
    import nqueens
    d = json.load(open(os.path.join(GOLDEN, "archive_digests.json")))["solutions"][str(N)]
    ld, rd, col, s = nqueens.gen_records_wide(N, 5)
    recs = np.zeros(len(s), nqueens.RECORD_DTYPE)
    recs["ld"] = ld & 0xFFFFFFFF; recs["rd"] = rd & 0xFFFFFFFF; recs["col"] = col & 0xFFFFFFFF; recs["startijkl"] = s
    total, sol = eng.exec_records(N, recs, want_solutions=True)
    assert total == d["sum"]
    assert solution_digest(s, ld, rd, col, sol) == d["sha256"]


@pytest.mark.parametrize("N", range(6, 17))
def test_per_record_counts_match_oracle_dynamic_preset(eng, oracle_mod, N):
    import nqueens
    recs = nqueens.gen_records(N)
    total, sol = eng.exec_records(N, recs, want_solutions=True)
    want = oracle_mod.exec_solutions(N, _o_records(oracle_mod, recs))
    assert np.array_equal(sol, want)
    assert total == oracle_mod.EXPECTED_TOTAL[N]


@pytest.mark.parametrize("N,preset", [(10, 4), (11, 6), (12, 7), (13, 4), (14, 6), (9, 7), (8, 6),
                                      (16, 4), (16, 6), (17, 7), (18, 5)])
def test_other_presets_match_oracle(eng, oracle_mod, N, preset):
    import nqueens
    recs = nqueens.gen_records(N, preset)
    total, sol = eng.exec_records(N, recs, want_solutions=True)
    want = oracle_mod.exec_solutions(N, _o_records(oracle_mod, recs))
    assert np.array_equal(sol, want)


@pytest.mark.parametrize("N", list(range(1, 20)))
def test_totals_known_answers(eng, oracle_mod, N):
    assert eng.count(N).total == oracle_mod.EXPECTED_TOTAL[N]


def test_total_n20(eng, oracle_mod):
    assert eng.count(20).total == oracle_mod.EXPECTED_TOTAL[20] == 39029188884


def test_total_n21_largest_configured_board(eng, oracle_mod):
    # 2,025,282 tasks at preset 6, one split level: about 7 s on one GB300
    r = eng.count(21)
    assert r.total == oracle_mod.EXPECTED_TOTAL[21] == 314666222712
    assert eng.last_run_info()[0] == 1


@pytest.mark.parametrize("N", [20, 21, 22, 24])
def test_large_board_sample_per_record(eng, oracle_mod, N):
    """A seeded sample of the N=20, 21 (preset 6), 22 and 24 (preset 7) task lists, per record against the
    oracle; N=24 runs the kernel form with u64 per-task counters."""
    import nqueens
    recs = nqueens.gen_records(N)
    idx = np.sort(np.random.default_rng(N).choice(len(recs), size=48, replace=False))
    sub = np.ascontiguousarray(recs[idx])
    del recs
    total, sol = eng.exec_records(N, sub, want_solutions=True)
    want = oracle_mod.exec_solutions(N, _o_records(oracle_mod, sub), threads=0)
    assert np.array_equal(sol, want)
    assert total == int(want.sum()) > 0


def test_headline_config_every_record(eng, oracle_mod):
    """The benchmark's workload, N=19 at preset 6: all 897,071 records against the oracle (about half a
    minute of oracle time on the host's cores)."""
    import nqueens
    recs = nqueens.gen_records(19)
    assert len(recs) == 897071
    total, sol = eng.exec_records(19, recs, want_solutions=True)
    want = oracle_mod.exec_solutions(19, _o_records(oracle_mod, recs), threads=0)
    assert int(np.count_nonzero(sol != want)) == 0
    assert total == int(want.sum()) == oracle_mod.EXPECTED_TOTAL[19]


def test_large_counts_per_record_low_preset(eng, oracle_mod):
    """N=21 at preset 4: a few records with large counts each, so the launch takes the u64 per-lane counters
    (sized from a bound on the count per queue item), split one and two levels, per record against the oracle."""
    import nqueens
    recs = nqueens.gen_records(21, 4)
    idx = np.sort(np.random.default_rng(21).choice(len(recs), size=4, replace=False))
    sub = np.ascontiguousarray(recs[idx])
    want = oracle_mod.exec_solutions(21, _o_records(oracle_mod, sub), threads=0)
    old = eng.get_config()
    try:
        for split in (1, 2):
            eng.set_config(64, 0, split)
            total, sol = eng.exec_records(21, sub, want_solutions=True)
            assert np.array_equal(sol, want), split
    finally:
        eng.set_config(*old)


def test_reference_dict_dropin(eng, oracle_mod):
    import nqueens
    _, _, cs, _ = nqueens.gen_constellations(11, set(), set(), [], 5)
    nqueens.exec_solutions(11, cs, True)
    assert sum(c["solutions"] for c in cs if c["solutions"] > 0) == 2680
    s = np.load(os.path.join(GOLDEN, "archive_small.npz"))["N11"]
    got = {(c["startijkl"], c["ld"], c["rd"], c["col"]): c["solutions"] for c in cs}
    for row in s.tolist():
        assert got[tuple(row[:4])] == row[4]


def test_device_resident_path(eng, oracle_mod):
    torch = pytest.importorskip("torch")
    import nqueens
    N = 15
    recs = nqueens.gen_records(N)
    d_rec = torch.from_numpy(recs.view(np.uint8).copy()).cuda()
    d_total = torch.zeros(1, dtype=torch.int64, device="cuda")
    d_sol = torch.zeros(len(recs), dtype=torch.int64, device="cuda")
    start_min = int((recs["startijkl"] >> 20).min())
    s = torch.cuda.Stream()
    for _ in range(2):
        eng.exec_device(N, d_rec.data_ptr(), len(recs), start_min, d_total.data_ptr(), d_sol.data_ptr(), s.cuda_stream)
        eng.sync()
        assert int(d_total.item()) == oracle_mod.EXPECTED_TOTAL[N]
    want = oracle_mod.exec_solutions(N, _o_records(oracle_mod, recs))
    assert np.array_equal(d_sol.cpu().numpy().view(np.uint64), want)
    p, k = eng.last_kernel_ms()
    assert p >= 0 and k > 0


def test_preset_too_deep_is_an_error(eng):
    import nqueens
    recs = nqueens.gen_records(6, 6)   # the reference raises on a negative shift for this preset
    with pytest.raises(nqueens.NQError) as ei:
        eng.exec_records(6, recs)
    assert ei.value.status == -6


def test_empty_and_single_record(eng, oracle_mod):
    import nqueens
    assert eng.exec_records(12, np.zeros(0, nqueens.RECORD_DTYPE))[0] == 0
    recs = nqueens.gen_records(12)
    want = oracle_mod.exec_solutions(12, _o_records(oracle_mod, recs))
    for i in (0, 7, len(recs) - 1):
        t, sol = eng.exec_records(12, recs[i:i + 1], want_solutions=True)
        assert t == int(want[i]) and int(sol[0]) == int(want[i])


def test_ragged_and_duplicated_records(eng, oracle_mod):
    """Records in any order, with duplicates: counts are per record."""
    import nqueens
    recs = nqueens.gen_records(13)
    rng = np.random.default_rng(7)
    idx = rng.integers(0, len(recs), size=5001)
    sub = recs[idx]
    t, sol = eng.exec_records(13, sub, want_solutions=True)
    want = oracle_mod.exec_solutions(13, _o_records(oracle_mod, sub))
    assert np.array_equal(sol, want) and t == int(want.sum())


@pytest.mark.parametrize("block", [64, 128, 256])
def test_launch_configs_agree(eng, oracle_mod, block):
    import nqueens
    eng.set_config(block, 0, -1)
    try:
        assert eng.count(16).total == oracle_mod.EXPECTED_TOTAL[16]
        eng.set_config(block, 37, -1)   # a grid that is not a multiple of anything
        assert eng.count(14).total == oracle_mod.EXPECTED_TOTAL[14]
    finally:
        eng.set_config(128, 0, -1)


@pytest.mark.parametrize("split", [0, 1, 2, 3])
def test_split_depths_per_record(eng, oracle_mod, split):
    """Per-record counts are the same whatever the split depth (subtask counts are summed per record)."""
    import nqueens
    eng.set_config(128, 0, split)
    try:
        for N in (8, 13, 15):
            recs = nqueens.gen_records(N)
            total, sol = eng.exec_records(N, recs, want_solutions=True)
            want = oracle_mod.exec_solutions(N, _o_records(oracle_mod, recs))
            assert np.array_equal(sol, want), (N, split)
            assert total == oracle_mod.EXPECTED_TOTAL[N]
        assert eng.count(17).total == oracle_mod.EXPECTED_TOTAL[17]
    finally:
        eng.set_config(128, 0, -1)


def _queens(rng, N, k):
    while True:
        rows = rng.choice(N, size=k, replace=False)
        cols = rng.integers(0, N, size=k)
        q = list(zip(rows.tolist(), cols.tolist()))
        if all(q[a][1] != q[b][1] and abs(q[a][0] - q[b][0]) != abs(q[a][1] - q[b][1])
               for a in range(k) for b in range(a + 1, k)):
            return q


@pytest.mark.parametrize("N", range(4, 14))
def test_completions_match_bruteforce(eng, oracle_mod, N):
    rng = np.random.default_rng(50 + N)
    for k in (0, 1, 2, 3, 4):
        q = _queens(rng, N, k)
        want = oracle_mod.completions(N, [r for r, _ in q], [c for _, c in q])
        assert eng.count_completions(N, q) == want, (N, q)


@pytest.mark.parametrize("N", [14, 15, 16, 17])
def test_completions_larger_boards(eng, oracle_mod, N):
    """One to eight pre-placed queens on larger boards (seeded rows and columns) against brute force."""
    rng = np.random.default_rng(700 + N)
    for k in ((1, 2, 3) if N < 17 else (2, 3)) + (6, 8):
        q = _queens(rng, N, k)
        want = oracle_mod.completions(N, [r for r, _ in q], [c for _, c in q])
        assert eng.count_completions(N, q) == want, (N, q)


def test_completion_edge_cases(eng, oracle_mod):
    assert eng.count_completions(8, [(0, 0), (1, 1)]) == 0          # attacking
    assert eng.count_completions(8, [(3, 3), (3, 5)]) == 0          # two queens in one row
    import nqueens
    with pytest.raises(nqueens.NQError):
        eng.count_completions(8, [(3, 3), (3, 3)])                  # the same queen twice is a bad argument
    with pytest.raises(nqueens.NQError):
        eng.count_completions(8, [(8, 0)])                          # off the board
    assert eng.count_completions(1, []) == 1
    assert eng.count_completions(3, []) == 0
    assert eng.count_completions(10, [(9, 0), (8, 2), (7, 4)]) == oracle_mod.completions(10, [9, 8, 7], [0, 2, 4])
    assert eng.count_completions(10, [(0, 9), (1, 7), (2, 5), (3, 3)]) == oracle_mod.completions(
        10, [0, 1, 2, 3], [9, 7, 5, 3])


def test_batch_mixed_jobs(eng, oracle_mod):
    import nqueens
    rng = np.random.default_rng(2026)
    jobs, want = [], []
    for _ in range(40):
        if rng.random() < 0.6:
            N = int(rng.integers(4, 15))
            jobs.append(nqueens.CountJob(N)); want.append(oracle_mod.EXPECTED_TOTAL[N])
        else:
            N = int(rng.integers(5, 13)); k = int(rng.integers(0, 5))
            q = _queens(rng, N, k)
            jobs.append(nqueens.CompletionJob(N, q))
            want.append(oracle_mod.completions(N, [r for r, _ in q], [c for _, c in q]))
    b = eng.batch(jobs)
    try:
        want = np.array(want, np.uint64)
        assert np.array_equal(b.run(use_graph=False), want)
        assert np.array_equal(b.run(use_graph=True), want)
        assert np.array_equal(b.run(use_graph=True), want)     # graph replay
        assert np.array_equal(b.run_plain(), want)
        b.submit(True)
        out = None
        for _ in range(10000):
            out = b.poll(1000)
            if out is not None:
                break
        assert out is not None and np.array_equal(out, want)
    finally:
        b.close()


def test_stack_shorter_than_a_task_is_an_error_not_a_partial_count(eng):
    """A start row claimed too deep sizes the stack too small: the call fails with NQ_ESTACK."""
    torch = pytest.importorskip("torch")
    import nqueens
    N = 12
    recs = nqueens.gen_records(N)
    d_rec = torch.from_numpy(recs.view(np.uint8).copy()).cuda()
    d_total = torch.zeros(1, dtype=torch.int64, device="cuda")
    eng.set_config(64, 0, 0)
    try:
        eng.exec_device(N, d_rec.data_ptr(), len(recs), 9, d_total.data_ptr())   # real start rows are 2..4
        with pytest.raises(nqueens.NQError) as ei:
            eng.sync()
        assert ei.value.status == -2
        eng.exec_device(N, d_rec.data_ptr(), len(recs), int((recs["startijkl"] >> 20).min()), d_total.data_ptr())
        eng.sync()
        assert int(d_total.item()) == 14200                   # the handle stays usable
    finally:
        eng.set_config(64, 0, -1)


def test_resumable_count_on_gpu(eng, oracle_mod, tmp_path):
    import nqueens
    from nqueens.checkpoint import exec_records_resumable
    recs = nqueens.gen_records(17)
    p = str(tmp_path / "p.tsv")
    counter = lambda n, r: eng.exec_records(n, r)[0]
    assert exec_records_resumable(counter, 17, recs, p, chunk=8192, stop_after=2) is None
    assert exec_records_resumable(counter, 17, recs, p, chunk=8192) == oracle_mod.EXPECTED_TOTAL[17]


def test_sync_waits_for_its_own_count_only(oracle_mod):
    """nq_sync waits on the handle's last count (an event), not on the whole device: two engines count
    device-resident records on their own streams and each collects its own total and status."""
    torch = pytest.importorskip("torch")
    import nqueens
    engines = [nqueens.Engine(0), nqueens.Engine(0)]
    try:
        outs = []
        for e, N in zip(engines, (16, 17)):
            recs = nqueens.gen_records(N)
            d_rec = torch.from_numpy(recs.view(np.uint8).copy()).cuda()
            d_tot = torch.zeros(1, dtype=torch.int64, device="cuda")
            s = torch.cuda.Stream()
            e.exec_device(N, d_rec.data_ptr(), len(recs), int((recs["startijkl"] >> 20).min()), d_tot.data_ptr(), 0,
                          s.cuda_stream)
            outs.append((N, d_rec, d_tot, s))
        for e, (N, _, d_tot, s) in zip(reversed(engines), reversed(outs)):
            e.sync()
            s.synchronize()
            assert int(d_tot.item()) == oracle_mod.EXPECTED_TOTAL[N]
        engines[0].sync()                      # nothing pending: waits for the handle's own stream only
    finally:
        for e in engines:
            e.close()


@pytest.mark.parametrize("N,chunk", [(12, 500), (17, 6000), (18, 100000)])
def test_chunked_whole_board_count(oracle_mod, N, chunk):
    """count() generates and counts the records chunk by chunk (bounded host memory for the largest boards):
    any chunk size gives the known total, and the chunks together hold every record once."""
    import nqueens
    e = nqueens.Engine(0)
    try:
        e.set_chunk_records(chunk)
        assert e.count(N).total == oracle_mod.EXPECTED_TOTAL[N]
        chunks, records = e.last_count_info()
        assert records == len(nqueens.gen_records(N))
        assert chunks >= max(2, records // (2 * chunk))
        e.set_chunk_records(0)
        assert e.count(N).total == oracle_mod.EXPECTED_TOTAL[N]
        assert e.last_count_info() == (1, records)
    finally:
        e.close()


def test_queue_order_leaves_counts_unchanged(eng, oracle_mod):
    """The DFS queue sorted largest-estimate-first on the device: the same per-record counts, split and
    unsplit."""
    import nqueens
    recs = nqueens.gen_records(15)
    want = oracle_mod.exec_solutions(15, _o_records(oracle_mod, recs))
    old = eng.get_config()
    try:
        eng.set_queue_order(1)
        for split in (0, 1, 2):
            eng.set_config(64, 0, split)
            total, sol = eng.exec_records(15, recs, want_solutions=True)
            assert np.array_equal(sol, want), split
    finally:
        eng.set_queue_order(0)
        eng.set_config(*old)


def test_count_starts_ranges_match_oracle(eng, oracle_mod):
    """count_starts(first, count) counts exactly the records whose start constellation lies in that range
    of start_constellations(N): each range against the oracle's per-record counts of those records, and
    an uneven partition adds up to the whole board."""
    import nqueens
    N = 14
    starts = nqueens.start_constellations(N)
    recs = nqueens.gen_records(N)
    per = oracle_mod.exec_solutions(N, _o_records(oracle_mod, recs))
    key = (recs["startijkl"] & 0xFFFFF).astype(np.int32)
    cuts = [0, 1, 7, 300, 301, 1000, len(starts)]
    acc = 0
    for a, b in zip(cuts[:-1], cuts[1:]):
        t = eng.count_starts(N, a, b - a)
        assert t == int(per[np.isin(key, starts[a:b])].sum()), (a, b)
        acc += t
    assert acc == oracle_mod.EXPECTED_TOTAL[N]
    assert eng.count_starts(N, 5, 0) == 0
    assert eng.count_starts(N, len(starts), 0) == 0
    for a, c in [(-1, 1), (0, len(starts) + 1), (len(starts), 1)]:
        with pytest.raises(nqueens.NQError) as ei:
            eng.count_starts(N, a, c)
        assert "start constellations" in str(ei.value)


@pytest.mark.parametrize("N,chunk", [(16, 500), (19, 4000)])
def test_count_resumable_by_start_ranges(oracle_mod, tmp_path, N, chunk):
    """A whole-board count cut at start-constellation boundaries, interrupted and resumed from its progress
    file, gives the known total and counts no range twice."""
    import nqueens
    from nqueens.checkpoint import count_resumable
    e = nqueens.Engine(0)
    p = str(tmp_path / "progress.tsv")
    try:
        assert count_resumable(e, N, p, chunk=chunk, stop_after=1) is None
        assert count_resumable(e, N, p, chunk=chunk) == oracle_mod.EXPECTED_TOTAL[N]
        lines = open(p).read().splitlines()[1:]
        n_starts = len(nqueens.start_constellations(N))
        assert len(lines) == (n_starts + chunk - 1) // chunk
        assert sorted(int(x.split("\t")[0]) for x in lines) == list(range(len(lines)))
    finally:
        e.close()


def test_cli_progress_resumes(tmp_path, capsys):
    from nqueens.cli import main
    p = str(tmp_path / "p.tsv")
    assert main(["15", "16", "--progress", p, "--chunk-starts", "300", "--stop-after", "2"]) == 0
    assert "stopped" in capsys.readouterr().out
    assert main(["15", "16", "--progress", p, "--chunk-starts", "300"]) == 0
    assert "2279184" in capsys.readouterr().out


def test_board_sharded_by_start_ranges_on_gpu(eng, oracle_mod):
    """Whole-board counts split over ranks by start-constellation chunks: one rank alone, and three ranks'
    chunk lists counted in turn on this GPU, give the known total."""
    import nqueens
    from nqueens.shard import board_chunks, count_board_sharded
    N = 17
    assert count_board_sharded(N, 0, 1, chunk=500, engine=eng) == oracle_mod.EXPECTED_TOTAL[N]
    n = len(nqueens.start_constellations(N))
    parts = [sum(eng.count_starts(N, a, c) for a, c in board_chunks(n, 300, r, 3)) for r in range(3)]
    assert sum(parts) == oracle_mod.EXPECTED_TOTAL[N] and min(parts) > 0
