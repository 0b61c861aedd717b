"""Chunked counting resumes from its progress file (CPU, the oracle counts each chunk)."""
import numpy as np
import pytest


def _oracle_counter(oracle_mod):
    def count(N, recs):
        o = oracle_mod.Records(recs["ld"].astype(np.uint64), recs["rd"].astype(np.uint64),
                               recs["col"].astype(np.uint64), recs["startijkl"].copy())
        return int(oracle_mod.exec_solutions(N, o, threads=2).sum()) if len(recs) else 0
    return count


def test_resume_after_interruption(tmp_path, oracle_mod):
    import nqueens
    from nqueens.checkpoint import exec_records_resumable
    N = 13
    recs = nqueens.gen_records(N)
    p = str(tmp_path / "progress.tsv")
    calls = []
    base = _oracle_counter(oracle_mod)

    def counter(n, r):
        calls.append(len(r))
        return base(n, r)

    assert exec_records_resumable(counter, N, recs, p, chunk=1000, stop_after=3) is None
    assert len(calls) == 3
    total = exec_records_resumable(counter, N, recs, p, chunk=1000)
    assert total == oracle_mod.EXPECTED_TOTAL[N]
    assert len(calls) == (len(recs) + 999) // 1000          # no chunk counted twice
    assert exec_records_resumable(counter, N, recs, p, chunk=1000) == total
    assert len(calls) == (len(recs) + 999) // 1000


def test_torn_line_is_recounted(tmp_path, oracle_mod):
    import nqueens
    from nqueens.checkpoint import exec_records_resumable
    N = 11
    recs = nqueens.gen_records(N)
    p = str(tmp_path / "progress.tsv")
    exec_records_resumable(_oracle_counter(oracle_mod), N, recs, p, chunk=500, stop_after=2)
    with open(p, "a") as f:
        f.write("2\t1000")                                   # an interrupted write
    assert exec_records_resumable(_oracle_counter(oracle_mod), N, recs, p, chunk=500) == oracle_mod.EXPECTED_TOTAL[N]


def test_progress_of_another_task_list_is_rejected(tmp_path, oracle_mod):
    import nqueens
    from nqueens.checkpoint import exec_records_resumable
    p = str(tmp_path / "progress.tsv")
    exec_records_resumable(_oracle_counter(oracle_mod), 10, nqueens.gen_records(10), p, chunk=300)
    with pytest.raises(ValueError):
        exec_records_resumable(_oracle_counter(oracle_mod), 11, nqueens.gen_records(11), p, chunk=300)


@pytest.mark.parametrize("N", range(9, 17))
def test_start_constellations_are_the_record_starts(oracle_mod, N):
    """The start list that count_starts partitions is the set of start constellations the oracle's
    generator expands (records carry their start in the low 20 bits of startijkl), ascending."""
    import nqueens
    st = nqueens.start_constellations(N)
    r = oracle_mod.gen_constellations(N, nqueens.select_dynamic_preset_queens(N))
    assert np.array_equal(st, np.unique(np.asarray(r.startijkl) & 0xFFFFF).astype(np.int32))
    assert (np.diff(st) > 0).all()


def test_start_constellations_small_and_bad_boards():
    import nqueens
    assert len(nqueens.start_constellations(6)) == 16
    for N in (5, 28):
        with pytest.raises(nqueens.NQError):
            nqueens.start_constellations(N)


class _StartsEngine:
    """count_starts by the oracle: the records of the range's starts, counted on the CPU."""

    def __init__(self, oracle_mod, N):
        import nqueens
        self.starts = nqueens.start_constellations(N)
        self.recs = nqueens.gen_records(N)
        self.per = oracle_mod.exec_solutions(N, oracle_mod.Records(
            self.recs["ld"].astype(np.uint64), self.recs["rd"].astype(np.uint64),
            self.recs["col"].astype(np.uint64), self.recs["startijkl"].copy()), threads=2)
        self.key = (self.recs["startijkl"] & 0xFFFFF).astype(np.int32)
        self.calls = []

    def count_starts(self, N, first, count, preset=None):
        self.calls.append((first, count))
        return int(self.per[np.isin(self.key, self.starts[first:first + count])].sum())


def test_count_resumable_by_start_ranges_cpu(tmp_path, oracle_mod):
    from nqueens.checkpoint import count_resumable
    N = 13
    e = _StartsEngine(oracle_mod, N)
    p = str(tmp_path / "progress.tsv")
    assert count_resumable(e, N, p, chunk=100, stop_after=4) is None
    assert len(e.calls) == 4
    assert count_resumable(e, N, p, chunk=100) == oracle_mod.EXPECTED_TOTAL[N]
    n_chunks = (len(e.starts) + 99) // 100
    assert len(e.calls) == n_chunks                          # no range counted twice
    assert sorted(e.calls) == [(a, min(100, len(e.starts) - a)) for a in range(0, len(e.starts), 100)]
    assert count_resumable(e, N, p, chunk=100) == oracle_mod.EXPECTED_TOTAL[N]
    assert len(e.calls) == n_chunks
    with pytest.raises(ValueError):                          # another chunk size never reuses the file
        count_resumable(e, N, p, chunk=50)


def test_cli_progress_needs_one_board(tmp_path, capsys):
    from nqueens.cli import main
    assert main(["15", "17", "--progress", str(tmp_path / "p.tsv")]) == 2
    assert not (tmp_path / "p.tsv").exists()


def test_count_resumable_time_limit(tmp_path, oracle_mod):
    """With a time limit no chunk starts unless 1.5 x the longest chunk so far still fits; the next run
    goes on from the progress file."""
    import time
    from nqueens.checkpoint import count_resumable
    N = 12
    e = _StartsEngine(oracle_mod, N)
    slow = e.count_starts

    def count_starts(*args):
        time.sleep(0.2)
        return slow(*args)
    e.count_starts = count_starts
    p = str(tmp_path / "progress.tsv")
    assert count_resumable(e, N, p, chunk=100, time_limit=0.5) is None
    assert 1 <= len(e.calls) <= 2
    e.count_starts = slow
    assert count_resumable(e, N, p, chunk=100) == oracle_mod.EXPECTED_TOTAL[N]
    assert len(e.calls) == (len(e.starts) + 99) // 100
