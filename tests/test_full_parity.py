"""Every record of the N=20 task list (preset 6) against the oracle (N=19, the benchmark's workload, is
in the default GPU suite: tests/test_gpu_parity.py).

Opt-in (minutes of oracle time on the host cores): NQ_FULL_PARITY=1 python -m pytest tests/test_full_parity.py -m gpu
"""
import os

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU"),
              pytest.mark.skipif(not os.environ.get("NQ_FULL_PARITY"), reason="opt-in: set NQ_FULL_PARITY=1")]


@pytest.mark.parametrize("N", [20])
def test_every_record(oracle_mod, N):
    import nqueens
    eng = nqueens.Engine(0)
    try:
        recs = nqueens.gen_records(N)
        total, sol = eng.exec_records(N, recs, want_solutions=True)
        o = oracle_mod.Records(recs["ld"].astype(np.uint64), recs["rd"].astype(np.uint64),
                               recs["col"].astype(np.uint64), recs["startijkl"].copy())
        want = oracle_mod.exec_solutions(N, o, threads=0)
        assert int(np.count_nonzero(sol != want)) == 0
        assert total == int(want.sum()) == oracle_mod.EXPECTED_TOTAL[N]
    finally:
        eng.close()
