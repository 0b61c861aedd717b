"""Autotuner host logic on the CPU: picks the fastest configuration per N, checks counts, saves and reloads."""
import json

import pytest

from nqueens import tune


class FakeEngine:
    """Timings with a known best configuration per N; counts constant unless told otherwise."""
    def __init__(self, best, flaky=False):
        self.best = best
        self.cfg = (64, 0, -1)
        self.flaky = flaky
        self.calls = 0

    def set_config(self, block, grid, split):
        self.cfg = (block, grid, split)

    def exec_records(self, N, recs):
        self.calls += 1
        return (N * 1000 + (self.calls if self.flaky else 0), None)

    def last_kernel_ms(self):
        b, g, s = self.cfg
        bb, bs = self.best
        return (0.01, 1.0 + abs(b - bb) / 64.0 + abs(s - bs))


def test_autotune_picks_fastest_and_round_trips(tmp_path, monkeypatch):
    monkeypatch.setattr(tune, "gen_records", lambda N: [0] * N)
    eng = FakeEngine(best=(128, 2))
    table = tune.autotune(eng, [12, 13], blocks=(64, 128, 256), splits=(0, 1, 2, 3), repeats=2, log=None)
    assert table["12"]["block"] == 128 and table["12"]["split"] == 2 and table["13"]["block"] == 128
    assert eng.cfg == (64, 0, -1)                                  # left at the defaults afterwards
    p = str(tmp_path / "t.json")
    tune.save(table, "GPU X", p)
    tune.save({"12": {"block": 64, "grid": 0, "split": 1, "ms": 1.0}}, "GPU Y", p)
    assert tune.load("GPU X", p) == table                         # other GPUs' tables are kept
    assert tune.load("GPU Y", p)["12"]["split"] == 1
    assert tune.load("GPU Z", p) is None
    assert tune.load("GPU X", str(tmp_path / "missing.json")) is None
    assert json.load(open(p))["GPU X"]["per_N"] == table


def test_autotune_rejects_changing_counts(monkeypatch):
    monkeypatch.setattr(tune, "gen_records", lambda N: [0] * N)
    with pytest.raises(RuntimeError):
        tune.autotune(FakeEngine(best=(64, 1), flaky=True), [12], blocks=(64,), splits=(1,), repeats=2, log=None)


def test_committed_table_is_well_formed():
    data = json.load(open(tune.DEFAULT_PATH))
    for gpu, entry in data.items():
        for N, cfg in entry["per_N"].items():
            assert 1 <= int(N) <= 27 and cfg["block"] in (64, 128, 256) and -1 <= cfg["split"] <= 3 and cfg["grid"] >= 0
