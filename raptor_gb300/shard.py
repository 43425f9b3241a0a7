"""Splitting a batch's rays across processes (one GPU each).

Rays are independent and the grid is replicated, so a batch shards by
contiguous ray ranges (raptor_gpu_render_range) with no communication while
rendering; the pieces are disjoint, so the full image is their sum and the
spectra add.  The adjoint shards the same way (raptor_gpu_vjp_range): every
gradient - the four scalars and the per-cell rho, u and ln Theta_e arrays -
is a sum over rays, so the gradient of the whole image is the sum of the
ranks' gradients.  With torch.distributed each merge is one
all_reduce(SUM); bench.py instead runs one independent image per rank (weak
scaling) and only synchronises its timers."""
from __future__ import annotations

import numpy as np

SCALARS = ("d_m_unit", "d_r_high", "d_r_low", "d_inclination")
FIELDS = ("d_rho", "d_u", "d_lnthetae")


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


def merge_grads(grads: dict, group=None) -> dict:
    """Sum one rank's gradients (the dict engine.Engine.vjp returns: four
    scalars, and per-cell arrays where present) over the ranks, in one
    all_reduce of a packed float64 buffer; returns the summed dict."""
    import torch
    import torch.distributed as dist
    fields = [k for k in FIELDS if k in grads]
    parts = [np.array([grads[k] for k in SCALARS], dtype=np.float64)]
    parts += [np.ascontiguousarray(grads[k], dtype=np.float64).ravel() for k in fields]
    buf = torch.from_numpy(np.concatenate(parts))
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    flat = buf.numpy()
    out = {k: float(flat[i]) for i, k in enumerate(SCALARS)}
    off = len(SCALARS)
    for k in fields:
        shape = np.shape(grads[k])
        n = int(np.prod(shape))
        out[k] = flat[off:off + n].reshape(shape).copy()
        off += n
    return out


def vjp_sharded(eng, img, dL_dI, precision, rank: int, world: int, group=None):
    """This rank's share of one image's VJP (its ray range), merged over the
    ranks: returns (the full image the VJP returns, the full gradients) on
    every rank."""
    begin, end = ray_range(img.width * img.height, world, rank)
    fimg, g = eng.vjp(img, dL_dI, precision, ray_begin=begin, ray_count=end - begin)
    return merge(fimg, group).numpy(), merge_grads(g, group)
