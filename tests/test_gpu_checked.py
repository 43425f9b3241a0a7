"""The bounds-checked build (libraptor_gpu_checked.so, -DRAPTOR_CHECKED):
every kernel checks the indices it computes - a ray's image and pixel, a
sample's grid cells, the output offset a ray writes, and the per-warp
sample-pool rings' fill, ticket lists and batch sizes - and a failed check
fails the call with RAPTOR_ERR_DEVICE.  The small parity cases run clean
under it (status OK, so no check failed) in every form and through every
kernel: the pooled and in-place FP64 kernels with one and five frequencies,
RK2, the log-polar camera, a mixed batch, a ray range and a trace, the mixed
and mixed-DF kernels, and the adjoints (pooled FP64 with one and three
frequencies, mixed, mixed-DF, each in one pass with its record tape and in
two passes; in-place FP64).  The checked build's images and gradients equal
the normal build's to rounding.
"""
import numpy as np
import pytest

from tests.parity import assert_fp64_parity

pytestmark = pytest.mark.gpu


def _cases(g64, g256):
    from raptor_gb300 import engine
    return [
        engine.image_desc(24, 20, [230e9], grid=g64, inclination=60.0),
        engine.image_desc(20, 16, [86e9, 140e9, 230e9, 345e9, 690e9], grid=g64, inclination=35.0),
        engine.image_desc(16, 16, [230e9], grid=g64, inclination=120.0, integrator=engine.RK2),
        engine.image_desc(16, 16, [230e9], grid=g256, inclination=17.0, camera=engine.CAM_LOG),
        [engine.image_desc(17, 9, [230e9], grid=g64, inclination=30.0),
         engine.image_desc(8, 12, [86e9, 345e9], grid=g256, inclination=150.0, m_unit=5e18),
         engine.image_desc(1, 1, [230e9], grid=g64, inclination=75.0)],
    ]


@pytest.mark.parametrize("no_pool", [0, 1], ids=["pooled", "in_place"])
def test_checked_build_renders_clean(torus64, torus256, no_pool):
    from raptor_gb300 import engine
    chk = engine.Engine(checked=True, no_sample_pool=no_pool)
    ref = engine.Engine(no_sample_pool=no_pool)
    try:
        ids = [(e.upload_grid(torus64.geom, torus64.prims), e.upload_grid(torus256.geom, torus256.prims))
               for e in (chk, ref)]
        for k, (dc, dr) in enumerate(zip(_cases(*ids[0]), _cases(*ids[1]))):
            for prec in (engine.PREC_FP64, engine.PREC_MIXED, engine.PREC_MIXED_DF):
                a, sa = chk.render(dc, prec)
                assert chk.last_status == 0, (k, prec)
                b, sb = ref.render(dr, prec)
                if prec == engine.PREC_FP64:
                    assert_fp64_parity(a, b, f"checked build, case {k}")
                else:
                    np.testing.assert_allclose(sa, sb, rtol=1e-6, err_msg=f"case {k}, form {prec}")
                assert chk.stats()["rays"] == ref.stats()["rays"]
        # a ray range and a trace
        d = _cases(*ids[0])[0]
        part, _ = chk.render(d, engine.PREC_FP64, ray_begin=37, ray_count=100)
        full, _ = ref.render(_cases(*ids[1])[0], engine.PREC_FP64)
        assert_fp64_parity(part[37:137], full[37:137], "checked range")
        rec = chk.trace_ray(d, 250)
        assert rec.shape[0] > 10
    finally:
        chk.close()
        ref.close()


@pytest.mark.parametrize("tape", [0, -1], ids=["one_pass", "two_pass"])
@pytest.mark.parametrize("prec,freqs", [(0, [230e9]), (0, [86e9, 230e9, 345e9]), (1, [230e9]), (2, [230e9])],
                         ids=["fp64", "fp64_3freq", "mixed", "mixed_df"])
def test_checked_build_adjoints_clean(torus64, prec, freqs, tape):
    from raptor_gb300 import engine
    out = {}
    for checked in (True, False):
        eng = engine.Engine(checked=checked, vjp_tape=tape)
        try:
            gid = eng.upload_grid(torus64.geom, torus64.prims)
            mk = lambda **o: engine.image_desc(32, 32, freqs, **dict(dict(grid=gid, inclination=60.0), **o))  # noqa: E731
            target, _ = eng.render(mk(inclination=62.0, m_unit=1.3e19), engine.PREC_FP64)
            img, _ = eng.render(mk(), engine.PREC_FP64)
            _, g = eng.vjp(mk(), img - target, prec)
            assert eng.last_status == 0
            out[checked] = g
        finally:
            eng.close()
    for k in ("d_m_unit", "d_r_high", "d_r_low", "d_inclination"):
        assert out[True][k] == pytest.approx(out[False][k], rel=1e-6), k
    for k in ("d_rho", "d_u", "d_lnthetae"):
        scale = float(np.abs(out[False][k]).max())
        assert float(np.abs(out[True][k] - out[False][k]).max()) <= 1e-6 * scale, k
