"""Data parallelism over GPUs: independent replicas.

Patches are independent (redux hands one patch per work request to each worker,
momfbdjob.cpp:363-376), so N GPUs solve disjoint sets of patches with no exchange on the
data path; only the timing is reduced across ranks (max) for reporting.
"""
from __future__ import annotations


def patch_range(n_total: int, rank: int, world: int):
    """Contiguous share of n_total patches for `rank` of `world` (sizes differ by <= 1)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    base, extra = divmod(n_total, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(values, device=None):
    """Element-wise maximum of a list of floats over all ranks (identity without a group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(values)
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()
