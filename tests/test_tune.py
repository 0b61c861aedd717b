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


def test_untuned_n_uses_defaults_not_previous_n(oracle_mod):
    """A count of an N the tuning table does not hold runs with the default configuration, not with the
    configuration the previous (tuned) N left behind."""
    import nqueens
    eng = nqueens.Engine(0)
    try:
        eng._tuning = {"14": {"block": 128, "grid": 0, "split": 3}}
        assert eng.count(14).total == oracle_mod.EXPECTED_TOTAL[14]
        assert eng.get_config() == (128, 0, 3)
        assert eng.count(13).total == oracle_mod.EXPECTED_TOTAL[13]
        assert eng.get_config() == (64, 0, -1)
    finally:
        eng.close()


def test_native_tuner_keeps_fastest_config_and_counts_stay_exact(oracle_mod):
    import nqueens
    eng = nqueens.Engine(0)
    try:
        b, s, ms = eng.tune_native(15, repeats=1)
        assert b in (64, 128, 256) and 0 <= s <= 3 and ms > 0
        assert eng.get_config() == (b, 0, s)
        assert eng.count(15).total == oracle_mod.EXPECTED_TOTAL[15]
        with pytest.raises(nqueens.NQError):
            eng.tune_native(5)                                 # the constellation path starts at N=6
    finally:
        eng.close()
