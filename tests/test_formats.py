"""Task and solution file formats against the reference's archived files (fixtures on CPU)."""
import json
import os

import numpy as np
import pytest

from conftest import REPO, gpu_available
from golden_util import solution_digest, task_digest

GOLDEN = os.path.join(REPO, "tests", "golden")


def test_task_file_round_trip_matches_archive_digest(tmp_path, oracle_mod):
    import nqueens
    from nqueens import formats
    d = json.load(open(os.path.join(GOLDEN, "archive_digests.json")))["tasks"]
    for N in (8, 12, 15):
        recs = nqueens.gen_records(N, 5)
        p = str(tmp_path / formats.task_file_name(N, 5))
        formats.save_tasks(p, recs)
        back = formats.load_tasks(p, require_done=True)
        assert np.array_equal(back, recs)
        assert os.path.getsize(p) == 16 * len(recs)
        assert task_digest(back["startijkl"], back["ld"], back["rd"], back["col"]) == d[str(N)]["sha256"]


def test_solution_file_round_trip_matches_archive(tmp_path, oracle_mod):
    from nqueens import formats
    s = np.load(os.path.join(GOLDEN, "archive_small.npz"))["N10"]
    arch = np.zeros(len(s), formats.SOLUTION_DTYPE)
    for i, k in enumerate(["startijkl", "ld", "rd", "col", "solutions"]):
        arch[k] = s[:, i]
    p = str(tmp_path / formats.solution_file_name(10, 5))
    formats.save_solutions(p, arch["ld"], arch["rd"], arch["col"], arch["startijkl"], arch["solutions"])
    back = formats.load_solutions(p)
    assert back.tobytes() == s.astype("<u8").tobytes()     # byte-identical to the reference's layout
    d = json.load(open(os.path.join(GOLDEN, "archive_digests.json")))["solutions"]["10"]
    assert solution_digest(back["startijkl"], back["ld"], back["rd"], back["col"], back["solutions"]) == d["sha256"]


def test_fill_from_solutions_and_cache_miss(tmp_path):
    import nqueens
    from nqueens import formats
    s = np.load(os.path.join(GOLDEN, "archive_small.npz"))["N9"]
    sol = np.zeros(len(s), formats.SOLUTION_DTYPE)
    for i, k in enumerate(["startijkl", "ld", "rd", "col", "solutions"]):
        sol[k] = s[:, i]
    _, _, cs, _ = nqueens.gen_constellations(9, set(), set(), [], 5)
    assert formats.fill_from_solutions(cs, sol) is None
    assert sum(c["solutions"] for c in cs) == 352
    cs.append({"ld": 1, "rd": 2, "col": 3, "startijkl": 4, "solutions": 0})
    assert formats.fill_from_solutions(cs, sol) == (4, 1, 2, 3)


def test_corrupt_files_are_rejected(tmp_path):
    import nqueens
    from nqueens import formats
    recs = nqueens.gen_records(9, 5)
    p = str(tmp_path / "t.bin")
    formats.save_tasks(p, recs)
    with open(p, "ab") as f:
        f.write(b"\x01\x02\x03")                      # truncated/extra bytes: size % 16 != 0
    with pytest.raises(formats.FormatError):
        formats.load_tasks(p)
    formats.save_tasks(p, recs)
    formats.write_done(p + ".done", len(recs) - 1)      # .done mismatch: an incomplete write
    with pytest.raises(formats.FormatError):
        formats.load_tasks(p, require_done=True)
    os.remove(p + ".done")
    with pytest.raises(formats.FormatError):
        formats.load_tasks(p, require_done=True)
    assert len(formats.load_tasks(p)) == len(recs)
    q = str(tmp_path / "s.bin")
    with open(q, "wb") as f:
        f.write(b"\x00" * 39)
    with pytest.raises(formats.FormatError):
        formats.load_solutions(q)



@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")
def test_cli_counts_a_task_file_and_writes_solutions(tmp_path, oracle_mod, capsys):
    import nqueens
    from nqueens import cli, formats
    N = 12
    recs = nqueens.gen_records(N)
    tp = str(tmp_path / formats.task_file_name(N, nqueens.select_dynamic_preset_queens(N)))
    sp = str(tmp_path / "solutions_out_v2.bin")
    formats.save_tasks(tp, recs)
    assert cli.main(["--tasks", tp, "--write-solutions", sp]) == 0
    assert f"total={oracle_mod.EXPECTED_TOTAL[N]}" in capsys.readouterr().out
    sol = formats.load_solutions(sp)
    want = oracle_mod.exec_solutions(N, oracle_mod.Records(recs["ld"].astype(np.uint64), recs["rd"].astype(np.uint64),
                                                           recs["col"].astype(np.uint64), recs["startijkl"].copy()))
    assert np.array_equal(sol["solutions"], want) and np.array_equal(sol["startijkl"], recs["startijkl"])


@pytest.mark.parametrize("N,block", [(9, 1), (13, 100), (16, 256), (19, 4096)])
def test_streamed_task_file_matches_archive(tmp_path, N, block):
    """The streamed writer appends a block of start constellations at a time; the finished file holds the
    same bytes as the whole list written at once, its .done the record count, and its records the
    reference's archived task list (digest of constellations_N{N}_5.bin)."""
    import nqueens
    from nqueens import formats
    d = json.load(open(os.path.join(GOLDEN, "archive_digests.json")))["tasks"]
    p = str(tmp_path / formats.task_file_name(N, 5))
    n = formats.stream_tasks(p, N, 5, starts_per_block=block)
    back = formats.load_tasks(p, require_done=True)
    assert n == len(back) == d[str(N)]["records"]
    assert task_digest(back["startijkl"], back["ld"], back["rd"], back["col"]) == d[str(N)]["sha256"]
    assert open(p, "rb").read() == nqueens.gen_records(N, 5).tobytes()


def test_records_of_start_ranges_partition_the_task_list():
    import nqueens
    N = 14
    n = len(nqueens.start_constellations(N))
    cuts = [0, 1, 2, 50, 51, 900, n]
    parts = [nqueens.gen_records_starts(N, a, b - a) for a, b in zip(cuts[:-1], cuts[1:])]
    assert np.concatenate(parts).tobytes() == nqueens.gen_records(N).tobytes()
    assert len(nqueens.gen_records_starts(N, n, 0)) == 0
    for a, c in [(-1, 1), (0, n + 1), (n, 1)]:
        with pytest.raises(nqueens.NQError):
            nqueens.gen_records_starts(N, a, c)
    with pytest.raises(nqueens.NQError):
        nqueens.gen_records_starts(N, 0, 5, preset=3)


def test_ensure_tasks_reuses_a_complete_file_and_rebuilds_others(tmp_path):
    import nqueens
    from nqueens import formats
    N = 12
    p = formats.ensure_tasks(N, 5, str(tmp_path))
    assert os.path.basename(p) == "constellations_N12_5.bin"
    want = nqueens.gen_records(N, 5).tobytes()
    assert open(p, "rb").read() == want
    mtime = os.stat(p).st_mtime_ns
    assert formats.ensure_tasks(N, 5, str(tmp_path)) == p and os.stat(p).st_mtime_ns == mtime   # cache hit
    with open(p, "r+b") as f:                                  # an interrupted write: shorter than .done says
        f.truncate(16 * 10)
    formats.ensure_tasks(N, 5, str(tmp_path))
    assert open(p, "rb").read() == want
    formats.write_done(p + ".done", 0)                          # a writer that never finished
    formats.ensure_tasks(N, 5, str(tmp_path))
    assert formats.read_done(p + ".done") == len(want) // 16


def test_cli_writes_a_task_file(tmp_path, capsys):
    import nqueens
    from nqueens import formats
    from nqueens.cli import main
    p = str(tmp_path / "constellations_N13_6.bin")
    assert main(["--write-tasks", p, "--n", "13", "--preset", "6"]) == 0
    assert "records=" in capsys.readouterr().out
    assert np.array_equal(formats.load_tasks(p, require_done=True), nqueens.gen_records(13, 6))
    assert main(["--write-tasks", p]) == 2
