"""Multi-GPU partitioning of one count: one process per GPU, no data-path collective.

Tasks are independent and the only exchange is one u64 per device (the
reference sums per-worker totals parsed from logs,
14Bit_codon_GPU/237Py_sum_worker_totals.py, after a static split
``chunk_index % worker_count == worker_id``, 356Py_savesp_narrow.py:5589-5590).
Here each rank takes the round-robin stripe ``records[rank::world]`` of the task
list -- records of similar cost spread evenly over ranks -- counts it on its own
GPU, and the totals are summed with one all_reduce of a single int64 on the host
side of torch.distributed (gloo or nccl).

``count_board_sharded`` splits a whole-board count the same way without any
task list: the board's start constellations are cut into chunks, rank r counts
chunks r, r + world, ... with ``Engine.count_starts`` (each generated on its own
host and counted on its own GPU), and one all_reduce sums the totals.
"""
from __future__ import annotations

from typing import Callable, Optional

import numpy as np


def shard_records(records: np.ndarray, rank: int, world: int) -> np.ndarray:
    """This rank's round-robin stripe of the task list."""
    if not (0 <= rank < world):
        raise ValueError(f"rank {rank} outside world of {world}")
    return records[rank::world]


def board_chunks(n_starts: int, chunk: int, rank: int, world: int):
    """This rank's [first, first + count) ranges of the start-constellation list: chunks rank, rank + world, ..."""
    if not (0 <= rank < world):
        raise ValueError(f"rank {rank} outside world of {world}")
    if chunk < 1:
        raise ValueError("chunk must be >= 1")
    return [(a, min(chunk, n_starts - a)) for a in range(rank * chunk, n_starts, world * chunk)]


def _sum_over_ranks(local: int, world: int, group) -> int:
    import torch
    import torch.distributed as dist
    if world == 1:
        return int(local)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([int(local)], dtype=torch.int64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return int(t.item())


def count_board_sharded(N: int, rank: int, world: int, preset: Optional[int] = None, chunk: int = 64,
                        engine=None, group=None) -> int:
    """Whole-board total of N over all ranks, each counting its chunks of start constellations with
    ``engine.count_starts`` (default: this process's GPU engine); every rank returns the same total."""
    from .engine import start_constellations
    if engine is None:
        from .engine import default_engine
        engine = default_engine()
    local = sum(engine.count_starts(N, a, c, preset) for a, c in board_chunks(len(start_constellations(N)), chunk,
                                                                                rank, world))
    return _sum_over_ranks(local, world, group)


def count_sharded(N: int, records: np.ndarray, rank: int, world: int,
                  counter: Optional[Callable[[int, np.ndarray], int]] = None, group=None) -> int:
    """Total count of all ranks' stripes.  ``counter(N, stripe) -> int`` counts one
    stripe (default: this process's GPU engine); every rank returns the same total."""
    stripe = shard_records(records, rank, world)
    if counter is None:
        from .engine import default_engine
        local = default_engine().exec_records(N, stripe)[0] if len(stripe) else 0
    else:
        local = int(counter(N, stripe))
    return _sum_over_ranks(local, world, group)
