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
