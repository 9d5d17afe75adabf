"""Dealing independent runs to ranks (one process per GPU).

A batched sweep of independent runs needs no communication: runs are dealt
whole to ranks, each rank advances its share in one context, and the only
collective is the max-over-ranks wall time of a timed region.  (The single
large run would shard as row slabs with a halo exchange; that path is not
built because every call here has one GPU.)
"""
from typing import List, Sequence


def deal_runs(zones: Sequence[int], world_size: int, rank: int) -> List[int]:
    """Indices of the runs this rank advances: longest-processing-time-first
    greedy assignment by zone count, so ranks get near-equal work.  The
    assignment depends only on `zones` and `world_size`."""
    if world_size < 1 or not (0 <= rank < world_size):
        raise ValueError("bad rank / world size")
    load = [0] * world_size
    owner = [0] * len(zones)
    for i in sorted(range(len(zones)), key=lambda k: (-zones[k], k)):
        r = min(range(world_size), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += zones[i]
    return [i for i in range(len(zones)) if owner[i] == rank]


def max_over_ranks(value: float, device=None) -> float:
    """Max of a scalar over all ranks of the default process group (identity
    when torch.distributed is not initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
