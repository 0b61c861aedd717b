"""Partition-and-sum across worker processes (world_size 2, gloo, CPU).

Each rank counts its round-robin stripe of the task list -- with the oracle as
the stand-in per-rank counter, since this host has no GPU -- and the ranks'
totals are summed by one all_reduce.  The sum must equal the board total, and
the stripes must cover every record exactly once.
"""
import os
import socket

import numpy as np
import pytest

from conftest import REPO


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, N, out_dir):
    import sys
    for p in (os.path.join(REPO, "n-queens_gb300"), os.path.join(REPO, "oracle")):
        sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    import nqueens
    import oracle
    from nqueens.shard import count_sharded, shard_records
    dist.init_process_group("gloo", rank=rank, world_size=world)
    recs = nqueens.gen_records(N)

    def counter(n, stripe):
        o = oracle.Records(stripe["ld"].astype(np.uint64), stripe["rd"].astype(np.uint64),
                           stripe["col"].astype(np.uint64), stripe["startijkl"].copy())
        return int(oracle.exec_solutions(n, o, threads=2).sum()) if len(stripe) else 0

    total = count_sharded(N, recs, rank, world, counter=counter)
    mine = shard_records(recs, rank, world)
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), mine["startijkl"])
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(str(total))
    dist.destroy_process_group()


@pytest.mark.parametrize("world,N", [(2, 12), (2, 13), (3, 11)])
def test_sharded_count_sums_to_total(tmp_path, oracle_mod, world, N):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(world, port, N, str(tmp_path)), nprocs=world, join=True, start_method="spawn")
    totals = [int(open(tmp_path / f"rank{r}.txt").read()) for r in range(world)]
    assert totals == [oracle_mod.EXPECTED_TOTAL[N]] * world
    import nqueens
    recs = nqueens.gen_records(N)
    got = np.sort(np.concatenate([np.load(tmp_path / f"rank{r}.npy") for r in range(world)]))
    assert np.array_equal(got, np.sort(recs["startijkl"]))


def test_shard_bounds():
    from nqueens.shard import shard_records
    recs = np.arange(10)
    assert list(shard_records(recs, 1, 3)) == [1, 4, 7]
    with pytest.raises(ValueError):
        shard_records(recs, 3, 3)


class _OracleStarts:
    """count_starts by the oracle: the records of the range's start constellations, counted on the CPU."""

    def __init__(self, oracle, N):
        self.o = oracle
        self.N = N
        self.calls = []

    def count_starts(self, N, first, count, preset=None):
        import nqueens
        self.calls.append((first, count))
        recs = nqueens.gen_records_starts(N, first, count, preset)
        if len(recs) == 0:
            return 0
        o = self.o.Records(recs["ld"].astype(np.uint64), recs["rd"].astype(np.uint64),
                           recs["col"].astype(np.uint64), recs["startijkl"].copy())
        return int(self.o.exec_solutions(N, o, threads=2).sum())


def _board_worker(rank, world, port, N, chunk, out_dir):
    import sys
    for p in (os.path.join(REPO, "n-queens_gb300"), os.path.join(REPO, "oracle")):
        sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    import oracle
    from nqueens.shard import count_board_sharded
    dist.init_process_group("gloo", rank=rank, world_size=world)
    eng = _OracleStarts(oracle, N)
    total = count_board_sharded(N, rank, world, chunk=chunk, engine=eng)
    with open(os.path.join(out_dir, f"board{rank}.txt"), "w") as f:
        f.write(f"{total} " + " ".join(f"{a}:{c}" for a, c in eng.calls))
    dist.destroy_process_group()


@pytest.mark.parametrize("world,N,chunk", [(2, 12, 50), (3, 13, 64)])
def test_board_sharded_by_start_ranges(tmp_path, oracle_mod, world, N, chunk):
    """Each rank counts its stripe of start-constellation chunks; one all_reduce gives every rank the board
    total, and the ranks' ranges cover the start list exactly once."""
    import torch.multiprocessing as mp
    import nqueens
    port = _free_port()
    mp.start_processes(_board_worker, args=(world, port, N, chunk, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    lines = [open(tmp_path / f"board{r}.txt").read().split() for r in range(world)]
    assert [int(x[0]) for x in lines] == [oracle_mod.EXPECTED_TOTAL[N]] * world
    covered = sorted(tuple(map(int, y.split(":"))) for x in lines for y in x[1:])
    n = len(nqueens.start_constellations(N))
    assert covered == [(a, min(chunk, n - a)) for a in range(0, n, chunk)]


def test_board_chunks_bounds():
    from nqueens.shard import board_chunks
    assert board_chunks(10, 3, 1, 2) == [(3, 3), (9, 1)]
    assert board_chunks(10, 3, 0, 2) == [(0, 3), (6, 3)]
    assert board_chunks(0, 3, 0, 2) == []
    with pytest.raises(ValueError):
        board_chunks(10, 3, 2, 2)
    with pytest.raises(ValueError):
        board_chunks(10, 0, 0, 2)
