"""Ray-range sharding across two gloo ranks on CPU: each rank renders its
share of a small image (with the oracle port standing in for a GPU) and the
all_reduce of the partial images equals the single-process image exactly."""
import os
import socket

import numpy as np
import pytest

from raptor_gb300 import shard


def test_ray_ranges_cover_exactly():
    for total in (0, 1, 7, 1000, 1024):
        for world in (1, 2, 3, 8):
            spans = [shard.ray_range(total, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == total
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(e - b for b, e in spans) - min(e - b for b, e in spans) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_path):
    import torch
    import torch.distributed as dist
    from oracle import port as oport
    from raptor_gb300 import synth
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    d = synth.make_torus(n1=64, n2=64)
    w = h = 12
    b, e = shard.ray_range(w * h, world, rank)
    part = np.zeros(w * h)
    vals, _ = oport.Scene(d.geom, d.prims, w, h, inclination=50.0).render([230e9], pixels=np.arange(b, e),
                                                                           nthreads=1)
    part[b:e] = vals[:, 0]
    full = shard.merge(torch.from_numpy(part)).numpy()
    if rank == 0:
        np.save(out_path, full)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_render_and_merge(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = str(tmp_path / "full.npy")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    from oracle import port as oport
    from raptor_gb300 import synth
    d = synth.make_torus(n1=64, n2=64)
    ref, _ = oport.Scene(d.geom, d.prims, 12, 12, inclination=50.0).render([230e9], nthreads=1)
    assert np.array_equal(np.load(out), ref[:, 0])


def _grad_worker(rank, world, port, out_path):
    """Each rank's gradients from its own ray range (per-ray contributions of
    the oracle port's image standing in for the adjoint, which needs a GPU),
    merged over the two ranks."""
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = _range_grads(*shard.ray_range(12 * 12, world, rank))
    full = shard.merge_grads(g)
    if rank == 0:
        np.savez(out_path, **{k: np.asarray(v) for k, v in full.items()})
    dist.barrier()
    dist.destroy_process_group()


def _range_grads(b, e):
    """Additive per-ray stand-in gradients of the rays [b, e) of a 12x12
    image: ray k adds its intensity I_k times fixed weights to the four
    scalars and to cells k mod 64 of a 8x8 grid."""
    from oracle import port as oport
    from raptor_gb300 import synth
    d = synth.make_torus(n1=64, n2=64)
    vals, _ = oport.Scene(d.geom, d.prims, 12, 12, inclination=50.0).render([230e9], pixels=np.arange(b, e),
                                                                           nthreads=1)
    g = {k: 0.0 for k in shard.SCALARS}
    fields = {k: np.zeros((8, 8)) for k in shard.FIELDS}
    for k, v in zip(range(b, e), vals[:, 0]):
        for q, name in enumerate(shard.SCALARS):
            g[name] += (q + 1) * v
        for q, name in enumerate(shard.FIELDS):
            fields[name].flat[k % 64] += (q + 2) * v
    g.update(fields)
    return g


def test_two_rank_gradient_merge(tmp_path):
    """merge_grads over two gloo ranks equals the single-process gradients of
    the whole image (the adjoint's gradients are sums over rays)."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = str(tmp_path / "grads.npz")
    mp.spawn(_grad_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    want = _range_grads(0, 144)
    for k in shard.SCALARS:
        assert float(got[k]) == pytest.approx(want[k], rel=1e-13), k
    for k in shard.FIELDS:
        np.testing.assert_allclose(got[k], want[k], rtol=1e-13, atol=0)
