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


def _common_keys(d, N=19):
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e"):
        assert k in d, k
    assert d["metric"] == f"N={N} DFS nodes/s" and d["unit"] == "nodes/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and "workload" in d["config"] and d["config"]["N"] == N


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(REPO, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_reference_arm_json_line():
    # a small board keeps the CPU suite quick; the driver runs the default N=19 workload
    d = _bench_line("--impl", "reference", "--n", "13", "--steps", "4", "--warmup", "1")
    _common_keys(d, 13)
    assert d["impl"] == "reference" and d["steps"] == 4
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["sample"]
    assert d["total"] == 73712                       # the timed slices together count the whole task list
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    # both arms print the same workload description
    assert d["config"] == _bench_module().bench_config(13)


def test_reference_arm_loads_no_engine_code():
    """The reference arm runs the oracle's generator and DFS only: the engine library is never loaded."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--n', '12', '--steps', '2', "
            "'--warmup', '1']\n"
            "try:\n    runpy.run_path('bench.py', run_name='__main__')\nexcept SystemExit:\n    pass\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libnqgpu' not in maps, 'engine library loaded'\n"
            "assert 'nqueens' not in sys.modules\n"
            "print('CLEAN')")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    assert "CLEAN" in out.stdout


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")
def test_our_arm_json_line():
    d = _bench_line("--steps", "1", "--warmup", "3", "--no-cpu", "--no-mix")
    _common_keys(d)
    assert d["total"] == 4968057848 and d["config"] == _bench_module().bench_config(19)
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert 0 < r["frac"] < 2 and r["peak"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] > 0 and d["e2e"]["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0 and "sm_mhz" in d["clocks"]
