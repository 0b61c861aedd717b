"""bench.py keeps its one-line JSON contract: each arm prints every key the driver reads."""
import json
import os
import subprocess
import sys

import pytest

from conftest import REPO, gpu_available


def _bench_line(*args):
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), *args], capture_output=True, text=True,
                         timeout=900, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    return json.loads(lines[0])


def _common_keys(d):
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e"):
        assert k in d, k
    assert d["metric"] == "N=19 DFS nodes/s" and d["unit"] == "nodes/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and "workload" in d["config"]


def test_reference_arm_json_line():
    d = _bench_line("--impl", "reference", "--steps", "1", "--warmup", "1", "--cpu-seconds", "1")
    _common_keys(d)
    assert d["impl"] == "reference" and d["steps"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")
def test_our_arm_json_line():
    d = _bench_line("--steps", "1", "--warmup", "3", "--no-cpu")
    _common_keys(d)
    assert d["n19_total"] == 4968057848
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert 0 < r["frac"] < 2 and r["peak"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] > 0 and d["e2e"]["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0 and "sm_mhz" in d["clocks"]
