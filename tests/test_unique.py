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


def test_unique_errors_carry_a_message(eng):
    """count_unique reports through the handle like every other call: the status and nq_last_error's text."""
    import nqueens
    with pytest.raises(nqueens.NQError) as e:
        eng.count_unique(3)
    assert e.value.status == -1 and "count_unique" in str(e.value)


def test_unique_runs_on_the_engines_device_and_stream():
    """Every engine counts on its own device with its own stream and buffers, whatever device the calling
    thread has current, and repeated calls reuse the handle's buffers."""
    torch = pytest.importorskip("torch")
    import nqueens
    n = torch.cuda.device_count()
    engines = [nqueens.Engine(d) for d in range(n)]
    try:
        for cur in range(n):
            torch.cuda.set_device(cur)
            for e in engines:
                for _ in range(2):
                    r = e.count_unique(12)
                    assert (r.unique, r.total) == (1787, 14200)
                assert torch.cuda.current_device() == cur
    finally:
        for e in engines:
            e.close()
        torch.cuda.set_device(0)
