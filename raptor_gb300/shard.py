"""Splitting a batch's rays across processes (one GPU each).

Rays are independent and the grid is replicated, so a batch shards by
contiguous ray ranges (raptor_gpu_render_range) with no communication while
rendering; the pieces are disjoint, so the full image is their sum and the
spectra add.  With torch.distributed the merge is one all_reduce(SUM) of the
image buffer; bench.py instead runs one independent image per rank (weak
scaling) and only synchronises its timers."""
from __future__ import annotations


def ray_range(total: int, world: int, rank: int) -> tuple[int, int]:
    """[begin, end) of rank's share of `total` rays, balanced to within one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(total, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def merge(partial, group=None):
    """Sum the per-rank partial images (zeros outside each rank's range) in
    place with torch.distributed; returns the full image."""
    import torch
    import torch.distributed as dist
    t = partial if isinstance(partial, torch.Tensor) else torch.from_numpy(partial)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t
