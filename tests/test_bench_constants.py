"""The frozen DFS node counts used by bench.py equal the oracle's node counter (small N)."""
import importlib.util
import os

import pytest

from conftest import REPO


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(REPO, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize("N", range(10, 17))
def test_frozen_node_counts(oracle_mod, N):
    b = _bench()
    rec = oracle_mod.gen_constellations(N, oracle_mod.preset_for(N))
    _, nodes = oracle_mod.exec_solutions(N, rec, want_nodes=True)
    assert int(nodes.sum()) == b.DFS_NODES[N]


def test_profile_figures_readable():
    b = _bench()
    assert b.read_traffic() > 0
    assert b.read_profile_figure("warp_instructions_per_launch") > 1e9
    assert 0 < b.read_profile_figure("alu_pipe_pct_of_peak") <= 100
    assert b.read_profile_figure("no_such_figure") is None
