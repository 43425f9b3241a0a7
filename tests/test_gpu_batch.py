"""Batched rendering: many images of uneven sizes, angles, frequencies,
M_unit and dumps in one persistent launch, replayed through a CUDA graph,
with the autotuned launch shape - against one render per image."""
import numpy as np
import pytest

from tests.parity import assert_fp64_parity

pytestmark = pytest.mark.gpu


def test_graph_batch_matches_single_renders():
    from raptor_gb300 import engine, workloads
    dumps = [d for d in workloads.batch_dumps(n=64)]
    sizes = [16] * 5 + [24] * 3 + [40]
    g_eng = engine.Engine(use_graph=1, autotune=1)
    p_eng = engine.Engine()
    gids = [g_eng.upload_grid(d.geom, d.prims) for d in dumps]
    pids = [p_eng.upload_grid(d.geom, d.prims) for d in dumps]
    assert gids == pids
    descs = workloads.batch_images(gids, seed=7, sizes=sizes)
    first, spec1 = g_eng.render(descs, engine.PREC_FP64)
    s1 = g_eng.stats()
    second, spec2 = g_eng.render(descs, engine.PREC_FP64)
    s2 = g_eng.stats()
    assert s1["graph_replayed"] == 0 and s2["graph_replayed"] == 1
    assert np.array_equal(first, second) and np.array_equal(spec1, spec2)
    assert s2["rays"] == sum(s * s for s in sizes)
    off = 0
    for d in descs:
        one, _ = p_eng.render(d, engine.PREC_FP64)
        assert_fp64_parity(second[off:off + one.size], one, "graph batch image")
        off += one.size
    # the graph is replayed with new descriptor contents of the same shape
    moved = workloads.batch_images(gids, seed=8, sizes=sizes)
    third, _ = g_eng.render(moved, engine.PREC_FP64)
    assert g_eng.stats()["graph_replayed"] == 1
    ref, _ = p_eng.render(moved, engine.PREC_FP64)
    assert_fp64_parity(third, ref, "replayed graph, new descriptors")
    g_eng.close()
    p_eng.close()
