"""Multi-GPU partitioning of one count: one process per GPU, no data-path collective.

Tasks are independent and the only exchange is one u64 per device (the
reference sums per-worker totals parsed from logs,
14Bit_codon_GPU/237Py_sum_worker_totals.py, after a static split
``chunk_index % worker_count == worker_id``, 356Py_savesp_narrow.py:5589-5590).
Here each rank takes the round-robin stripe ``records[rank::world]`` of the task
list -- records of similar cost spread evenly over ranks -- counts it on its own
GPU, and the totals are summed with one all_reduce of a single int64 on the host
side of torch.distributed (gloo or nccl).
"""
from __future__ import annotations

from typing import Callable, Optional

import numpy as np


def shard_records(records: np.ndarray, rank: int, world: int) -> np.ndarray:
    """This rank's round-robin stripe of the task list."""
    if not (0 <= rank < world):
        raise ValueError(f"rank {rank} outside world of {world}")
    return records[rank::world]


def count_sharded(N: int, records: np.ndarray, rank: int, world: int,
                  counter: Optional[Callable[[int, np.ndarray], int]] = None, group=None) -> int:
    """Total count of all ranks' stripes.  ``counter(N, stripe) -> int`` counts one
    stripe (default: this process's GPU engine); every rank returns the same total."""
    import torch
    import torch.distributed as dist
    stripe = shard_records(records, rank, world)
    if counter is None:
        from .engine import default_engine
        local = default_engine().exec_records(N, stripe)[0] if len(stripe) else 0
    else:
        local = int(counter(N, stripe))
    if world == 1:
        return int(local)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([int(local)], dtype=torch.int64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return int(t.item())
