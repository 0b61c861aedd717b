"""Unique counts (symmetry method) on the GPU against the oracle and the known table."""
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


@pytest.fixture(scope="module")
def eng():
    import nqueens
    e = nqueens.Engine(0)
    yield e
    e.close()


@pytest.mark.parametrize("N", range(4, 14))
def test_unique_matches_oracle(eng, oracle_mod, N):
    r = eng.count_unique(N)
    assert (r.unique, r.total) == oracle_mod.unique_symmetry(N)


@pytest.mark.parametrize("N", range(14, 22))   # N=21: about 14 s on one GB300
def test_unique_known_answers(eng, oracle_mod, N):
    r = eng.count_unique(N)
    assert r.unique == oracle_mod.EXPECTED_UNIQUE[N]
    assert r.total == oracle_mod.EXPECTED_TOTAL[N]


def test_unique_bad_n(eng):
    import nqueens
    for N in (3, 28):
        with pytest.raises(nqueens.NQError):
            eng.count_unique(N)
