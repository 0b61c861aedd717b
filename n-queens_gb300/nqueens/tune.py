"""Autotuner for the DFS launch: threads per block, split depth and grid, per N.

For each N the tuner times the whole count (prepare + split + DFS, device time
from CUDA events on the launching stream) over a grid of candidates and keeps
the fastest; the table is keyed by the GPU's name and saved as JSON next to
this module (``tuning.json``).  ``Engine`` applies a saved table automatically
when the GPU's name matches.  The stack depth needs no tuning: every launch
sizes its shared-memory stack to the deepest task it holds.  The queue is
claimed one warp-aggregated atomic per refill; the split depth sets how fine
the queued work items are, which is the queue granularity knob.

    python -m nqueens.tune [N ...] [--blocks 64 128 256] [--splits 0 1 2 3]
"""
from __future__ import annotations

import argparse
import json
import os
import time
from typing import Dict, Iterable, Optional

from .engine import Engine, gen_records

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_PATH = os.path.join(HERE, "tuning.json")


def time_config(eng: Engine, N: int, recs, block: int, split: int, grid: int = 0, repeats: int = 3) -> float:
    """Best device ms of prepare+split+DFS for one configuration (the count is checked each run)."""
    eng.set_config(block, grid, split)
    total0, _ = eng.exec_records(N, recs)
    best = float("inf")
    for _ in range(repeats):
        total, _ = eng.exec_records(N, recs)
        if total != total0:
            raise RuntimeError(f"N={N}: count changed between runs ({total} != {total0})")
        p, d = eng.last_kernel_ms()
        best = min(best, p + d)
    return best


def autotune(eng: Engine, Ns: Iterable[int], blocks=(64, 128, 256), splits=(0, 1, 2, 3), grids=(0,),
             repeats: int = 3, log=print) -> Dict[str, dict]:
    table: Dict[str, dict] = {}
    for N in Ns:
        recs = gen_records(N)
        best = None
        for b in blocks:
            for s in splits:
                for g in grids:
                    ms = time_config(eng, N, recs, b, s, g, repeats)
                    if log:
                        log(f"N={N} block={b} split={s} grid={g}: {ms:.3f} ms")
                    if best is None or ms < best[0]:
                        best = (ms, b, s, g)
        table[str(N)] = {"block": best[1], "split": best[2], "grid": best[3], "ms": round(best[0], 4)}
    eng.set_config(64, 0, -1)
    return table


def save(table: Dict[str, dict], name: str, path: str = DEFAULT_PATH) -> None:
    data = {}
    if os.path.exists(path):
        with open(path) as f:
            data = json.load(f)
    data[name] = {"when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()), "per_N": table}
    with open(path, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)


def load(name: str, path: str = DEFAULT_PATH) -> Optional[Dict[str, dict]]:
    try:
        with open(path) as f:
            return json.load(f).get(name, {}).get("per_N")
    except (OSError, ValueError):
        return None


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m nqueens.tune")
    ap.add_argument("N", nargs="*", type=int, default=[14, 15, 16, 17, 18, 19, 20])
    ap.add_argument("--blocks", nargs="+", type=int, default=[64, 128, 256])
    ap.add_argument("--splits", nargs="+", type=int, default=[0, 1, 2, 3])
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--out", default=DEFAULT_PATH)
    a = ap.parse_args(argv)
    eng = Engine(0, auto_tune=False)
    table = autotune(eng, a.N, a.blocks, a.splits, repeats=a.repeats)
    save(table, eng.device_name(), a.out)
    print(json.dumps(table, indent=1))
    eng.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
