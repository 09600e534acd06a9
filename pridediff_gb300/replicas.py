"""Replicas on several GPUs of one node.

The DD operators need no collective on their data path: slices (and the
instances of an uneven batch) are independent, so N GPUs run N replicas, each
on its own contiguous shard of the slices.  The only cross-rank operation is
the max over ranks of a timing (the slowest replica sets the job's time).

This module holds that host logic; ``bench.py --gpus N`` uses it under
torchrun with NCCL, and the CPU tests run it with two gloo ranks.
"""
from __future__ import annotations

from typing import Sequence, Tuple


def shard_bounds(n: int, rank: int, world: int) -> Tuple[int, int]:
    """[lo, hi) of rank's contiguous shard of n items; sizes differ by at most one."""
    if world <= 0 or not 0 <= rank < world or n < 0:
        raise ValueError("need 0 <= rank < world and n >= 0")
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def shard(items: Sequence, rank: int, world: int) -> list:
    lo, hi = shard_bounds(len(items), rank, world)
    return list(items[lo:hi])


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank float over the initialised process group (the
    value itself when there is none or it has one rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
