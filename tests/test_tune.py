"""Autotuner: picks a configuration per N, saves and reloads it, counts stay exact."""
import json

import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


def test_autotune_small_grid_round_trip(tmp_path, oracle_mod):
    import nqueens
    from nqueens import tune
    eng = nqueens.Engine(0, auto_tune=False)
    try:
        table = tune.autotune(eng, [11, 13], blocks=(64, 128), splits=(0, 2), repeats=1, log=None)
        assert set(table) == {"11", "13"}
        for v in table.values():
            assert v["block"] in (64, 128) and v["split"] in (0, 2) and v["ms"] > 0
        p = str(tmp_path / "t.json")
        tune.save(table, eng.device_name(), p)
        assert tune.load(eng.device_name(), p) == json.load(open(p))[eng.device_name()]["per_N"]
        eng._tuning = table                 # what Engine(auto_tune=True) does with a saved table
        for N in (11, 13):
            assert eng.count(N).total == oracle_mod.EXPECTED_TOTAL[N]
    finally:
        eng.close()
