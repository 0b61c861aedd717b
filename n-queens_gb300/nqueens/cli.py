"""Command line: the reference's per-N table, on the GB300 engine.

    python -m nqueens [nmin nmax] [--repeat R] [--split D] [--block B] [--unique]
    python -m nqueens --tasks constellations_N19_6.bin [--write-solutions solutions_N19_6_v2.bin]

prints, like the reference's main() (14Bit_codon_GPU/356Py_savesp_narrow.py:5899-6046),

     N:             Total           Unique         hh:mm:ss.ms
    19:        4968057848                0         0:00:00.152    ok

for N in range(nmin, nmax), with "ok" / "ng(got!=expected)" against the
reference's known-answer table (356Py_savesp_narrow.py:5775).  Unique is 0 on
the constellation path, as in the reference, unless --unique is given.
--repeat runs each count R times (the last one is printed), which is how
profiles/ captures a warm kernel.

--progress FILE counts one board (nmin, with nmax = nmin + 1) in chunks of
start constellations, appending each chunk's total to FILE and skipping the
chunks already there, so a count too long for one run is finished by rerunning
the same command (--stop-after C ends a run after C new chunks, --time-limit S
before a chunk that would end past S seconds).

--write-tasks FILE with --n (and --preset) writes the board's task list as the
reference's constellations_N{N}_{P}.bin with its .done sidecar, streamed a block
of start constellations at a time (host only, no GPU).

--tasks counts one of the reference's cached task files (16-byte records,
N taken from the file name or --n) and --write-solutions writes the
per-record counts as the reference's 40-byte solutions_*_v2.bin cache.  The
task file holds only the low 32 bits of each mask, so the written cache is
keyed by those: it is found again by a reference run that also loads its
constellations from the task file, not by one that generates them afresh
with full-width masks.  For full-width keys use --n with --regenerate, which
generates the board's constellations (nqueens.gen_records_wide) instead of
reading a task file.
"""
from __future__ import annotations

import argparse
import datetime as dt
import sys

from .engine import Engine

# Known totals, 356Py_savesp_narrow.py:5775 (index = N).
EXPECTED = [0, 1, 0, 0, 2, 10, 4, 40, 92, 352, 724, 2680, 14200, 73712, 365596, 2279184, 14772512, 95815104,
            666090624, 4968057848, 39029188884, 314666222712, 2691008701644, 24233937684440, 227514171973736,
            2207893435808352, 22317699616364044, 234907967154122528]


def _fmt(td: dt.timedelta) -> str:
    return str(td)[:-3] if td.microseconds else str(td) + ".000"


def _count_task_file(a) -> int:
    import os
    import re

    from . import formats
    m = re.search(r"_N(\d+)_", os.path.basename(a.tasks))
    N = a.n or (int(m.group(1)) if m else 0)
    if not 6 <= N <= 27:
        print(f"{a.tasks}: give the board size with --n (6..27)", file=sys.stderr)
        return 2
    return _count_records(a, N, formats.load_tasks(a.tasks), None, a.tasks)


def _count_records(a, N, recs, wide, name) -> int:
    import numpy as np

    from . import formats
    eng = Engine(a.device, block=a.block, split=a.split)
    try:
        t0 = dt.datetime.now()
        total, sol = eng.exec_records(N, recs, want_solutions=bool(a.write_solutions))
        el = dt.datetime.now() - t0
    finally:
        eng.close()
    status = "ok" if N < len(EXPECTED) and EXPECTED[N] == total else "(no known answer for this task set)"
    print(f"{name}: N={N} records={len(recs)} total={total} {_fmt(el)} {status}")
    if a.write_solutions:
        if wide is not None:                  # full-width masks, as the reference's fresh constellations carry
            ld, rd, col, sijkl = wide
        else:                                 # the task file's 32-bit masks
            ld, rd, col = (recs[k].astype(np.uint64) for k in ("ld", "rd", "col"))
            sijkl = recs["startijkl"]
        formats.save_solutions(a.write_solutions, ld, rd, col, sijkl.astype(np.uint64), sol)
    return 0


def _count_regenerated(a) -> int:
    from .engine import gen_records, gen_records_wide
    N = a.n
    if not 6 <= N <= 27:
        print("--regenerate needs --n (6..27)", file=sys.stderr)
        return 2
    preset = a.preset or None
    return _count_records(a, N, gen_records(N, preset), gen_records_wide(N, preset), f"N={N} generated")


def _count_with_progress(a) -> int:
    from .checkpoint import count_resumable
    N = a.nmin
    if a.nmax != N + 1 or not 6 <= N <= 27:
        print("--progress counts one board: give nmin and nmax = nmin + 1, 6 <= nmin <= 27", file=sys.stderr)
        return 2
    eng = Engine(a.device, block=a.block, split=a.split)
    try:
        t0 = dt.datetime.now()
        total = count_resumable(eng, N, a.progress, a.preset or None, a.chunk_starts, a.stop_after,
                                log=lambda m: print(m, file=sys.stderr, flush=True), time_limit=a.time_limit)
        el = dt.datetime.now() - t0
    finally:
        eng.close()
    if total is None:
        print(f"{N:2d}: stopped ({_fmt(el)}); rerun to continue from {a.progress}")
        return 0
    status = "ok" if N < len(EXPECTED) and EXPECTED[N] == total else f"ng({total}!={EXPECTED[N]})"
    print(f"{N:2d}:{total:18d}{0:17d}{_fmt(el):>21s}    {status}")
    return 0 if status == "ok" else 1


def _write_tasks(a) -> int:
    from . import formats
    N = a.n
    if not 6 <= N <= 27:
        print("--write-tasks needs --n (6..27)", file=sys.stderr)
        return 2
    t0 = dt.datetime.now()
    n = formats.stream_tasks(a.write_tasks, N, a.preset or None)
    print(f"{a.write_tasks}: N={N} records={n} {_fmt(dt.datetime.now() - t0)}")
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m nqueens", description=__doc__.split("\n")[0])
    ap.add_argument("nmin", nargs="?", type=int, default=5)
    ap.add_argument("nmax", nargs="?", type=int, default=20, help="exclusive upper bound, as range()")
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--split", type=int, default=-1)
    ap.add_argument("--block", type=int, default=64)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--unique", action="store_true", help="also count unique solutions (symmetry method)")
    ap.add_argument("--tasks", help="count a reference task file constellations_N{N}_{P}.bin")
    ap.add_argument("--n", type=int, default=0, help="board size of --tasks when its name does not give it")
    ap.add_argument("--write-solutions", help="with --tasks or --regenerate: write the per-record counts as a v2 "
                                              "solutions file")
    ap.add_argument("--regenerate", action="store_true",
                    help="with --n: generate the constellations (full-width masks) instead of reading --tasks")
    ap.add_argument("--preset", type=int, default=0,
                    help="with --regenerate, --progress or --write-tasks: preset queens (0: the dynamic preset)")
    ap.add_argument("--write-tasks", help="with --n: write the task list to this .bin file (no count)")
    ap.add_argument("--progress", help="count board nmin resumably, keeping per-chunk totals in this file")
    ap.add_argument("--chunk-starts", type=int, default=64, help="with --progress: start constellations per chunk")
    ap.add_argument("--stop-after", type=int, default=None, help="with --progress: stop after this many new chunks")
    ap.add_argument("--time-limit", type=float, default=None,
                    help="with --progress: start no chunk that would end past this many seconds")
    a = ap.parse_args(argv)
    if a.write_tasks:
        return _write_tasks(a)
    if a.progress:
        return _count_with_progress(a)
    if a.regenerate:
        return _count_regenerated(a)
    if a.tasks:
        return _count_task_file(a)
    eng = Engine(a.device, block=a.block, split=a.split)   # the defaults keep the autotuned table
    rc = 0
    try:
        print(" N:             Total           Unique         hh:mm:ss.ms")
        for N in range(a.nmin, a.nmax):
            for _ in range(max(1, a.repeat)):
                t0 = dt.datetime.now()
                r = eng.count_unique(N) if a.unique and N >= 4 else eng.count(N)
                el = dt.datetime.now() - t0
            status = "ok" if N < len(EXPECTED) and EXPECTED[N] == r.total else f"ng({r.total}!={EXPECTED[N]})"
            if status != "ok":
                rc = 1
            print(f"{N:2d}:{r.total:18d}{r.unique:17d}{_fmt(el):>21s}    {status}", flush=True)
    finally:
        eng.close()
    return rc


if __name__ == "__main__":
    sys.exit(main())
