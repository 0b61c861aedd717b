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
