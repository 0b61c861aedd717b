"""libnqgpu.so on a CPU-only host: exports, host generator, task schedules.

No kernel runs here.  The schedule tests replay, in Python, the per-node
step of dfs_kernel (nq_kernels.cu) over the schedule words the library's own
host code derives for each record, and compare the counts with the oracle
record for record: `replay` in the reference's terms (used columns, an
explicit depth), `replay_lane` as the kernel's lane runs it (free-column
frames, depth from their popcount, the sentinel frame).
"""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REPO
from golden_util import canonical_order, task_digest

M32 = 0xFFFFFFFF


@pytest.fixture(scope="session")
def nq():
    import nqueens
    from nqueens import _lib
    here = os.path.join(REPO, "n-queens_gb300")
    import importlib.util
    spec = importlib.util.spec_from_file_location("nq_build", os.path.join(here, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    _lib.lib()
    return nqueens


def header_functions():
    src = open(os.path.join(REPO, "include", "nqueens_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nq_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(nq):
    from nqueens import _lib
    names = header_functions()
    assert len(names) >= 20
    L = _lib.lib()
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(_lib.SIGNATURES), "ctypes binding and header disagree"


def test_version_and_strerror(nq):
    from nqueens import _lib
    assert b"sm_103a" in _lib.lib().nq_version()
    assert _lib.lib().nq_strerror(_lib.NQ_ESTACK)


@pytest.mark.parametrize("N", range(6, 22))
def test_generator_matches_archived_tasks(nq, N):
    import json
    d = json.load(open(os.path.join(REPO, "tests", "golden", "archive_digests.json")))["tasks"][str(N)]
    r = nq.gen_records(N, 5)
    assert len(r) == d["records"]
    assert task_digest(r["startijkl"], r["ld"], r["rd"], r["col"]) == d["sha256"]


@pytest.mark.parametrize("N,preset", [(n, p) for n in range(6, 17) for p in (4, 6, 7)] + [(18, 6), (19, 6), (20, 6)])
def test_generator_matches_oracle(nq, oracle_mod, N, preset):
    try:
        o = oracle_mod.gen_constellations(N, preset)
    except ValueError:
        from nqueens import NQError
        with pytest.raises(NQError):
            nq.gen_records_wide(N, preset)
        return
    ld, rd, col, s = nq.gen_records_wide(N, preset)
    assert len(s) == len(o)
    a = canonical_order(s, ld, rd, col)
    b = canonical_order(o.startijkl, o.ld, o.rd, o.col)
    assert np.array_equal(s[a], o.startijkl[b])
    assert np.array_equal(ld[a], o.ld[b]) and np.array_equal(rd[a], o.rd[b]) and np.array_equal(col[a], o.col[b])


def test_gen_constellations_dropin_signature(nq):
    ijkl, cache, cs, p = nq.gen_constellations(10, set(), set(), [], 5)
    assert p == 5 and len(cs) == 1007 and isinstance(ijkl, set) and len(cache) == 0
    assert set(cs[0]) == {"ld", "rd", "col", "startijkl", "solutions"}


def test_presets(nq):
    assert [nq.select_dynamic_preset_queens(n) for n in (5, 17, 18, 21, 22, 25, 27)] == [5, 5, 6, 6, 7, 8, 8]


# --- replay of dfs_kernel's node step -----------------------------------------------------------
def replay(root, info, words, wide):
    T = info & 31
    wexp = (info >> 5) & 3
    cnt = (info >> 7) & 1
    N = (info >> 8) & 31
    if T == 31:
        return cnt << wexp, 0
    bm = (1 << N) - 1
    ld, rd, col, avail = root
    stack = []
    d = 0
    nodes = 0
    while True:
        if avail == 0:
            if not stack:
                break
            ld, rd, col, avail, d = stack.pop()
        bit = avail & (-avail & M32)
        avail ^= bit
        nodes += 1
        if wide:
            x, ra = words[d]
            s = x & 31; la = (x >> (32 - s)) if s else 0
            fc, term, tall = x & (1 << 5), x & (1 << 6), x & (1 << 7)
        else:                        # compact word: s in bits 0-4, RA << s at bits N-1..N, FC bit 28, LA on top
            w = words[d]
            s = w & 31; la = w >> (32 - s); ra = (w & (3 << (N - 1))) >> s
            fc, term, tall = w & (1 << 28), d == T, 0
        nld = (((ld | bit) << s) & M32) | la
        nrd = ((rd | bit) >> s) | ra
        ncol = col | bit
        nf = bm & ~(nld | nrd | ncol)
        if fc and (bm & ~((((nld << 1) & M32) | (nrd >> 1) | ncol))) == 0:
            nf = 0
        if term:                     # SQd2B: LA bit 0 of the word already removed column 0
            cnt += 1 if (nf != 0 or tall) else 0
        elif nf:
            if avail:
                stack.append((ld, rd, col, avail, d))
            ld, rd, col, avail, d = nld, nrd, ncol, nf, d + 1
    return cnt << wexp, nodes


def schedule_of(rec, N):
    from nqueens import _lib
    r = _lib.nq_record(int(rec["ld"]), int(rec["rd"]), int(rec["col"]), int(rec["startijkl"]))
    root = np.zeros(4, np.uint32)
    info = np.zeros(1, np.uint32)
    words = np.zeros(32, np.uint32)
    n = _lib.lib().nq_debug_task_schedule(N, r, _lib.p32(root), _lib.p32(info), _lib.p32(words), 32)
    assert n >= 0
    return [int(x) for x in root], int(info[0]), [int(x) for x in words[:n]]


@pytest.mark.parametrize("N,preset", [(n, p) for n in range(6, 13) for p in (4, 5, 6, 7)] + [(13, 5), (14, 5)])
def test_schedule_replay_matches_oracle(nq, oracle_mod, N, preset):
    try:
        o = oracle_mod.gen_constellations(N, preset)
        if len(o) == 0:
            return
        sol, nodes = oracle_mod.exec_solutions(N, o, threads=1, want_nodes=True)
    except ValueError:
        pytest.skip("the reference raises for this preset (negative shift)")
    rec = np.zeros(len(o), nq.RECORD_DTYPE)
    rec["ld"] = o.ld & M32; rec["rd"] = o.rd & M32; rec["col"] = o.col & M32; rec["startijkl"] = o.startijkl
    for i in range(len(o)):
        root, info, words = schedule_of(rec[i], N)
        got, nd = replay(root, info, words, wide=False)
        assert got == int(sol[i]), (i, rec[i])
        assert nd <= int(nodes[i])   # pruning may only remove work


@pytest.mark.parametrize("N", [10, 12, 13])
def test_lookahead_on_every_sound_word(nq, oracle_mod, N):
    """The schedule builder sets the look-ahead flag on every word whose child step is one row and not a
    tall terminal (the rule that makes the prune count-preserving), and the replay with those flags still
    gives the oracle's per-record counts with fewer or equal nodes."""
    o = oracle_mod.gen_constellations(N, 5)
    sol, nodes = oracle_mod.exec_solutions(N, o, threads=1, want_nodes=True)
    rec = np.zeros(len(o), nq.RECORD_DTYPE)
    rec["ld"] = o.ld & M32; rec["rd"] = o.rd & M32; rec["col"] = o.col & M32; rec["startijkl"] = o.startijkl
    flagged = fewer = 0
    for i in range(len(o)):
        root, info, words = schedule_of(rec[i], N)
        T = info & 31
        if T == 31:
            continue
        for d in range(T):
            child = words[d + 1]
            if (child & 31) == 1:    # the child steps one row (compact words are never tall)
                assert words[d] & (1 << 28), (i, d, hex(words[d]), hex(child))
                flagged += 1
        got, nd = replay(root, info, words, wide=False)
        assert got == int(sol[i])
        fewer += nd < int(nodes[i])
    assert flagged > 0 and fewer > 0


def test_completion_lookahead_flags(nq):
    """Completion schedules: look-ahead on every word whose child is a one-row, non-tall step; never on the
    parent of the tall last row."""
    for queens in ([(0, 1)], [(2, 5), (7, 3)], [(5, 0)]):
        for root, info, w in completion_tasks(12, queens):
            T = info & 31
            if T == 31:
                continue
            for d in range(T):
                x1 = w[d + 1][0]
                sound = (x1 & 31) == 1 and not (x1 & (1 << 7))
                assert bool(w[d][0] & (1 << 5)) == sound, (queens, d)


@pytest.mark.parametrize("N,preset", [(n, p) for n in (8, 11, 14, 17) for p in (4, 5, 6, 7)])
def test_compact_word_fields_do_not_overlap(nq, oracle_mod, N, preset):
    """Compact schedule words step 1, 2 or 3 rows (bits 0-4), keep RA << s inside bits N-1..N and LA in the
    top s bits, clear of the look-ahead flag (bit 28): the DFS kernel's two funnel shifts read the fields in
    place, exact only under these bounds (the prepare kernel rejects a task whose op would not fit)."""
    try:
        o = oracle_mod.gen_constellations(N, preset)
    except ValueError:
        pytest.skip("the reference raises for this preset (negative shift)")
    rec = np.zeros(len(o), nq.RECORD_DTYPE)
    rec["ld"] = o.ld & M32; rec["rd"] = o.rd & M32; rec["col"] = o.col & M32; rec["startijkl"] = o.startijkl
    seen = set()
    ram = 3 << (N - 1)
    for i in range(0, len(o), max(1, len(o) // 4000)):
        _, info, words = schedule_of(rec[i], N)
        for w in words:
            s = w & 31
            assert 1 <= s <= 3, (i, hex(w))
            la_region = (M32 >> (32 - s)) << (32 - s)
            middle = w & ~31 & ~(1 << 28) & ~la_region & M32
            assert middle & ~ram == 0, (i, hex(w))          # RA << s only at bits N-1..N
            seen.add(s)
    assert not seen or 1 in seen


def _funnel_l(lo, hi, n):
    n &= 31
    return ((((hi << 32) | lo) << n) >> 32) & M32


def _funnel_r(lo, hi, n):
    n &= 31
    return (((hi << 32) | lo) >> n) & M32


@pytest.mark.parametrize("N", [9, 13, 16])
def test_funnel_shift_child_masks(nq, oracle_mod, N):
    """The DFS kernel's child rows from two funnel shifts of the compact word equal the reference's
    ((ld | bit) << s) | LA and ((rd | bit) >> s) | RA, for masks with garbage above the board in ld and
    high bits in rd (both occur: ld's shifted-out queens, rd's pre-loaded diagonals)."""
    o = oracle_mod.gen_constellations(N, 5)
    rec = np.zeros(len(o), nq.RECORD_DTYPE)
    rec["ld"] = o.ld & M32; rec["rd"] = o.rd & M32; rec["col"] = o.col & M32; rec["startijkl"] = o.startijkl
    rng = np.random.default_rng(N)
    ram = 3 << (N - 1)
    checked = 0
    for i in range(0, len(o), max(1, len(o) // 500)):
        _, info, words = schedule_of(rec[i], N)
        for w in words:
            s = w & 31; la = w >> (32 - s); ra = (w & ram) >> s
            for x, y in rng.integers(0, 1 << 32, size=(8, 2), dtype=np.uint64).tolist():
                assert _funnel_l(w, x, w) == ((x << s) & M32) | la
                assert _funnel_r(y | (w & ram), 0, w) == (y >> s) | ra
                checked += 1
    assert checked > 0


def completion_tasks(N, queens, min_tasks=64):
    from nqueens import _lib
    k = len(queens)
    rows = (ctypes.c_int * max(1, k))(*[q[0] for q in queens])
    cols = (ctypes.c_int * max(1, k))(*[q[1] for q in queens])
    L = _lib.lib()
    fixed = np.zeros(1, np.uint64)
    n = L.nq_debug_completion_tasks(N, k, rows, cols, min_tasks, None, None, None, 32, 0, _lib.p64(fixed))
    assert n >= 0
    roots = np.zeros(max(1, n) * 4, np.uint32)
    infos = np.zeros(max(1, n), np.uint32)
    words = np.zeros(max(1, n) * 32 * 2, np.uint32)
    n2 = L.nq_debug_completion_tasks(N, k, rows, cols, min_tasks, _lib.p32(roots), _lib.p32(infos), _lib.p32(words),
                                     32, n, None)
    assert n2 == n
    out = [([0, 0, 0, 0], 31 | (int(fixed[0]) << 7), [])] if fixed[0] else []
    for i in range(n):
        T = int(infos[i]) & 31
        w = [(int(words[(i * 32 + d) * 2]), int(words[(i * 32 + d) * 2 + 1])) for d in range(T + 1)]
        out.append(([int(x) for x in roots[i * 4:i * 4 + 4]], int(infos[i]), w))
    return out


def random_queens(rng, N, k):
    while True:
        rows = rng.choice(N, size=k, replace=False)
        cols = rng.integers(0, N, size=k)
        q = list(zip(rows.tolist(), cols.tolist()))
        ok = all(q[a][1] != q[b][1] and abs(q[a][0] - q[b][0]) != abs(q[a][1] - q[b][1])
                 for a in range(k) for b in range(a + 1, k))
        if ok:
            return q


@pytest.mark.parametrize("N", range(1, 11))
def test_completion_replay_matches_bruteforce(nq, oracle_mod, N):
    rng = np.random.default_rng(1000 + N)
    cases = [[]] + [random_queens(rng, N, k) for k in (1, 1, 2, 2, 3, 4) if k < N]
    if N >= 6:   # queens on consecutive rows and in the corners exercise multi-row steps and injections
        cases.append([(1, 0), (2, N - 1)])
        cases.append([(N - 1, 1), (N - 2, N - 1), (0, 2)] if N > 6 else [(0, 1), (2, 0)])
    for q in cases:
        if len(set(r for r, _ in q)) != len(q):
            continue
        want = oracle_mod.completions(N, [r for r, _ in q], [c for _, c in q])
        got = sum(replay(root, info, w, wide=True)[0] for root, info, w in completion_tasks(N, q))
        assert got == want, (N, q)


def test_completion_attacking_queens_have_no_tasks(nq):
    assert completion_tasks(8, [(0, 0), (1, 1)]) == []
    assert completion_tasks(8, [(0, 3), (5, 3)]) == []


def test_completion_full_board(nq, oracle_mod):
    q = [(2, 0), (0, 1), (3, 2), (1, 3)]       # a full 4-queens solution
    t = completion_tasks(4, q)
    assert sum(replay(root, info, w, wide=True)[0] for root, info, w in t) == 1 == oracle_mod.completions(
        4, [r for r, _ in q], [c for _, c in q])


def _popc(x):
    return bin(x).count("1")


def replay_lane(root, info, words, wide):
    """One DFS lane of dfs_kernel as it runs on the GPU: frames {ld, rd, fr, avail} with fr the row's free
    columns, the depth taken from popc(fr), the child's rows from the funnel shifts of the word with '+' for
    '|', the terminal test on popc(fr) (compact words), and a sentinel frame {~0, ~0, root fr, 0} under the
    stack.  Asserts the invariants the kernel relies on: every candidate is a free column and in neither
    diagonal (so '-' and '+' are exact), and every word the lane reads lies within its schedule.  Returns
    (weighted count, steps)."""
    T = info & 31
    wexp = (info >> 5) & 3
    cnt = (info >> 7) & 1
    N = (info >> 8) & 31
    if T == 31:
        return cnt << wexp, 0
    bm = (1 << N) - 1
    ram = 3 << (N - 1)
    ld, rd, col, avail = root
    fr = bm & ~col
    R = _popc(fr)
    assert avail & ~fr == 0
    tf = R - T
    stack = [(M32, M32, fr, 0)]                 # the sentinel
    steps = 0
    while True:
        if avail == 0:
            if not stack:
                break
            ld, rd, fr, avail = stack.pop()
        pf = _popc(fr)
        d = R - pf
        assert 0 <= d <= T                      # the word read stays inside the lane's schedule
        act = avail != 0
        bit = avail & (-avail & M32)
        avail -= bit
        if act:
            steps += 1
            assert bit & fr and not bit & ld and not bit & rd
        if wide:
            x, ra = words[d]
            s = x & 31
            nld = ((((ld + bit) & M32) << s) | (x >> (32 - s) if s else 0)) & M32
            nrd = (((rd + bit) & M32) >> s) | ra
            term, fc, tall = bool(x & (1 << 6)), bool(x & (1 << 5)), bool(x & (1 << 7))
        else:
            w = words[d]
            s = w & 31
            nld = ((((ld + bit) & M32) << s) | (w >> (32 - s) if s else 0)) & M32
            nrd = (((rd + bit) & M32) | (w & ram)) >> s
            term, fc, tall = pf == tf, bool(w & (1 << 28)), False
        free = fr - bit
        nf = free & ~(nld | nrd) & M32
        ahead = free & ~((((nld + nld) & M32) | (nrd >> 1))) & M32
        live = nf != 0
        hit = (act and live and term) or (act and term and tall) if wide else (live and term)
        cnt += 1 if hit else 0
        desc = (act if wide else True) and live and not term and not (fc and ahead == 0)
        if desc and avail:
            stack.append((ld, rd, fr, avail))
        if desc:
            ld, rd, fr, avail = nld, nrd, free, nf
    return cnt << wexp, steps


@pytest.mark.parametrize("N,preset", [(n, p) for n in range(6, 12) for p in (4, 5, 6, 7)] + [(12, 5), (13, 6)])
def test_lane_replay_matches_oracle(nq, oracle_mod, N, preset):
    """The kernel's lane state machine (free-column frames) gives every record's count, visits the same
    steps as the reference-semantics replay, and keeps its invariants."""
    try:
        o = oracle_mod.gen_constellations(N, preset)
        if len(o) == 0:
            return
        sol = oracle_mod.exec_solutions(N, o, threads=1)
    except ValueError:
        pytest.skip("the reference raises for this preset (negative shift)")
    rec = np.zeros(len(o), nq.RECORD_DTYPE)
    rec["ld"] = o.ld & M32; rec["rd"] = o.rd & M32; rec["col"] = o.col & M32; rec["startijkl"] = o.startijkl
    for i in range(len(o)):
        root, info, words = schedule_of(rec[i], N)
        got, steps = replay_lane(root, info, words, wide=False)
        assert got == int(sol[i]), (i, rec[i])
        assert steps == replay(root, info, words, wide=False)[1]


@pytest.mark.parametrize("N", range(4, 11))
def test_lane_replay_of_completion_tasks(nq, oracle_mod, N):
    rng = np.random.default_rng(2000 + N)
    for q in [[]] + [random_queens(rng, N, k) for k in (1, 2, 2, 3) if k < N]:
        want = oracle_mod.completions(N, [r for r, _ in q], [c for _, c in q])
        got = sum(replay_lane(root, info, w, wide=True)[0] for root, info, w in completion_tasks(N, q))
        assert got == want, (N, q)


def test_exec_solutions_rejects_cpu_path(nq):
    with pytest.raises(ValueError):
        nq.exec_solutions(8, [{"ld": 0, "rd": 0, "col": 0, "startijkl": 0, "solutions": 0}], use_gpu=False)



def test_entry_points_reject_a_null_handle(nq):
    """Calls that need a handle return NQ_EINVAL for a null one (no device is touched)."""
    import ctypes
    from nqueens import _lib
    L = _lib.lib()
    b, s, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
    assert L.nq_tune(None, 15, 1, ctypes.byref(b), ctypes.byref(s), ctypes.byref(ms)) == _lib.NQ_EINVAL
    t = np.zeros(1, np.uint64)
    assert L.nq_count(None, 10, 0, _lib.p64(t)) == _lib.NQ_EINVAL
    assert L.nq_set_config(None, 64, 0, -1) == _lib.NQ_EINVAL


@pytest.mark.parametrize("N", [8, 16, 20])
def test_presets_below_four_are_rejected(nq, N):
    """The start constellations already hold three or four queens, and the reference's presets are 4..8:
    a preset below 4 is rejected at once with NQ_EPRESET (it used to run the expansion for seconds at N=16
    and past a minute at N=18), by the generator and by the whole-board sizing call."""
    import time
    from nqueens import NQError
    for preset in (1, 2, 3):
        t0 = time.perf_counter()
        with pytest.raises(NQError) as e:
            nq.gen_records(N, preset)
        assert e.value.status == -6 and time.perf_counter() - t0 < 1.0
    with pytest.raises(NQError) as e:
        nq.engine.job_device_bytes(nq.CountJob(N, 3), 152)
    assert e.value.status == -6
