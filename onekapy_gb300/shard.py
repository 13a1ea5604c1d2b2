"""Realization sharding across ranks (one process per GPU).

Realizations are independent, and each one is drawn from its own Philox
counter (realization index), so a rank that takes the contiguous index range
[first, first + n) draws exactly the realizations a single process would.
Each rank chronicles its range into its own int32 counts; an integer
all-reduce (SUM) of the count grids and of the registered totals gives the
single-process result bit for bit, in any partition.
"""
from __future__ import annotations

import torch


def shard_range(nreal: int, rank: int, world: int) -> tuple[int, int]:
    """(first, count) of rank's contiguous share of nreal realizations."""
    if world < 1 or not (0 <= rank < world) or nreal < 0:
        raise ValueError("bad shard arguments")
    base, extra = divmod(nreal, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def reduce_counts(counts: torch.Tensor, registered: torch.Tensor | None = None, group=None):
    """Sum the int32 count grids (and registered totals) of all ranks in place."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return counts, registered
    dist.all_reduce(counts, op=dist.ReduceOp.SUM, group=group)
    if registered is not None:
        dist.all_reduce(registered, op=dist.ReduceOp.SUM, group=group)
    return counts, registered
