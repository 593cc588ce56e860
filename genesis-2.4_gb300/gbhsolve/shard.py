"""Neuron sharding across ranks (one process per GPU).

Neurons are independent block-diagonal systems, so a model shards by
contiguous neuron ranges with no exchange on the data path; only results
(step time, spike counts, losses) are reduced at the end.
"""
from __future__ import annotations


def shard_range(n_items: int, rank: int, world: int):
    """Contiguous [lo, hi) share of n_items for rank (sizes differ by <= 1)."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    base, extra = divmod(n_items, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def reduce_max(value: float, dist=None) -> float:
    """Max over ranks (the job's time is its slowest rank's)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(values, dist=None):
    if dist is None:
        return values
    import torch
    t = torch.as_tensor(values, dtype=torch.float64).clone()
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.numpy()
