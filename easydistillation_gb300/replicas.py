"""Replica bookkeeping for several GPUs of one node.

Timeslices are independent (each ``calc(t)`` reads only its own links and
eigenvectors), so N GPUs run N replicas that split the timeslices
round-robin; the only cross-rank operations are a barrier and a max of the
timed region (no collective on the data path)."""

from __future__ import annotations

from typing import List

import torch


def timeslices_for_rank(Lt: int, rank: int, world: int) -> List[int]:
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("need 0 <= rank < world")
    return list(range(rank, Lt, world))


def max_over_ranks(value: float, device=None) -> float:
    """Max of a host float over the default process group (identity without one)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
