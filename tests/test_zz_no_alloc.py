"""raptor_gpu_render_noalloc: the render entry point for callers that
cannot allocate device memory (an application that owns all device memory
through its own pool, or a loop that must not take cudaMalloc's lock and
device synchronisation).  The caller brings the grid and the outputs in its
own device memory; the entry point keeps its scratch in a fixed device array.

Checked through the C ABI against raptor_gpu_render on the same inputs, for
two calls in a row (the second must not see the first call's leftovers in the
shared scratch), at the FP64 parity bar the other GPU tests use.  This file
sorts last so a first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from tests.parity import assert_fp64_parity

pytestmark = pytest.mark.gpu


def _noalloc_lib():
    from raptor_gb300 import engine
    lib = engine.load()
    lib.raptor_gpu_render_noalloc.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(engine.GridGeomC),
                                              ctypes.POINTER(engine.ImageDesc), ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p]
    lib.raptor_gpu_render_noalloc.restype = ctypes.c_int
    return lib


@pytest.mark.parametrize("freqs", [([230e9], [230e9]), ([86e9, 230e9, 345e9], [140e9])],
                         ids=["one_frequency", "three_and_one_frequencies"])
def test_noalloc_render_matches_render(torus64, freqs):
    """Two images per call; the second case gives the first image three
    frequencies, so the spectrum map has image and frequency halves of
    different lengths and the render takes the multi-frequency kernel."""
    torch = pytest.importorskip("torch")
    from raptor_gb300 import engine
    lib = _noalloc_lib()

    # the reference result through the ordinary entry point
    eng = engine.Engine()
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    descs = [engine.image_desc(20, 14, freqs[0], grid=gid, inclination=60.0),
             engine.image_desc(9, 11, freqs[1], grid=gid, inclination=150.0, m_unit=4e19)]
    want, want_spec = eng.render(descs, engine.PREC_FP64)
    eng.close()
    n0 = 20 * 14 * len(freqs[0])

    # the caller's own device memory: grid as [n1][n2][8] cells, outputs
    g = torus64.geom
    cells = torch.from_numpy(np.ascontiguousarray(np.moveaxis(torus64.prims, 0, -1))).cuda()
    out = torch.empty(want.size, dtype=torch.float64, device="cuda")
    spec = torch.empty(want_spec.size, dtype=torch.float64, device="cuda")
    geom = engine.GridGeomC(g.n1, g.n2, g.startx1, g.startx2, g.dx1, g.dx2, g.a, g.hslope, g.R0)
    arr = (engine.ImageDesc * 2)(*descs)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out.fill_(-1.0)
        spec.fill_(-1.0)
        torch.cuda.synchronize()
        rc = lib.raptor_gpu_render_noalloc(0, cells.data_ptr(), ctypes.byref(geom), arr, 2, out.data_ptr(),
                                           spec.data_ptr(), stream)
        assert rc == 0, f"call {call}: status {rc}"
        assert torch.cuda.current_device() == 0
        got = out.cpu().numpy()
        assert_fp64_parity(got[:n0], want[:n0], f"noalloc image 0, call {call}")
        assert_fp64_parity(got[n0:], want[n0:], f"noalloc image 1, call {call}")
        np.testing.assert_allclose(spec.cpu().numpy(), want_spec, rtol=1e-6)

    # a batch beyond the stated maximum is refused, and nothing is launched
    big = (engine.ImageDesc * 17)(*([descs[0]] * 17))
    rc = lib.raptor_gpu_render_noalloc(0, cells.data_ptr(), ctypes.byref(geom), big, 17, out.data_ptr(),
                                       spec.data_ptr(), stream)
    assert rc == -6
