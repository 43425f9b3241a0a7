"""The kappa-distribution emission model (RAPTOR_EMISSION_KAPPA): the fits of
j_nu.c:28-106, kappa = 3.5, in place of the thermal ones, rendered by the
FP64 form and compared with the oracle port, whose kappa functions equal
the reference's own (tests/test_oracle.py), at the FP64 parity bar of
tests/parity.py; rendered by the mixed and mixed-DF forms (the FP32 fits of
kappa.cuh) and compared with the FP64 form at the mixed forms' flux bar.
The kappa adjoints: the FP64 one against central differences
(tests/test_gpu_vjp.py), the mixed forms' against the FP64 one."""
import numpy as np
import pytest

from tests.parity import FLUX_RTOL_MIXED, assert_fp64_parity, pixel_errors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from raptor_gb300 import engine
    e = engine.Engine()
    yield e
    e.close()


@pytest.mark.parametrize("n,w,h,freqs,incl,camera", [
    (64, 24, 20, [230e9], 60.0, 0),
    (64, 17, 13, [86e9, 230e9, 690e9], 35.0, 0),
    (256, 48, 40, [230e9], 75.0, 0),
    (256, 32, 24, [345e9], 20.0, 1),
])
def test_kappa_image_matches_port(eng, torus64, torus256, n, w, h, freqs, incl, camera):
    from oracle import port
    from raptor_gb300 import engine
    d = torus64 if n == 64 else torus256
    gid = eng.upload_grid(d.geom, d.prims)
    desc = engine.image_desc(w, h, freqs, grid=gid, inclination=incl, camera=camera,
                             emission=engine.EMISSION_KAPPA)
    img, spec = eng.render(desc, engine.PREC_FP64)
    st = eng.stats()
    assert st["rays"] == w * h and st["n_nonfinite"] == 0
    ref, _ = port.Scene(d.geom, d.prims, w, h, inclination=incl, camera=camera, emission=1).render(freqs)
    assert np.count_nonzero(ref) > 0.2 * ref.size
    assert_fp64_parity(img, ref.ravel(), f"kappa {n} {w}x{h} {len(freqs)} freq")
    np.testing.assert_allclose(spec, ref.sum(axis=0), rtol=1e-6)
    # a different image from the thermal model's
    thermal, _ = eng.render(engine.image_desc(w, h, freqs, grid=gid, inclination=incl, camera=camera),
                            engine.PREC_FP64)
    assert not np.allclose(thermal, img, rtol=1e-3, atol=0.0)


def test_kappa_pooled_equals_in_place(torus64):
    """The pooled and in-place FP64 kernels run the same kappa arithmetic."""
    from raptor_gb300 import engine
    out = []
    for nsp in (0, 1):
        e = engine.Engine(no_sample_pool=nsp)
        gid = e.upload_grid(torus64.geom, torus64.prims)
        out.append(e.render(engine.image_desc(32, 32, [230e9, 345e9], grid=gid, inclination=50.0,
                                              emission=engine.EMISSION_KAPPA), engine.PREC_FP64)[0])
        e.close()
    np.testing.assert_allclose(out[0], out[1], rtol=1e-12, atol=0)


@pytest.mark.parametrize("prec", [1, 2], ids=["mixed", "mixed_df"])
@pytest.mark.parametrize("n,w,h,freqs,incl,camera", [
    (64, 48, 40, [230e9], 60.0, 0),
    (256, 40, 32, [86e9, 230e9, 690e9], 35.0, 0),
    (256, 32, 24, [345e9], 20.0, 1),
])
def test_kappa_mixed_forms_match_fp64(eng, torus64, torus256, prec, n, w, h, freqs, incl, camera):
    """The FP32 kappa fits against the FP64 form's: every frequency's flux
    within the mixed forms' 1e-4, and the summed absolute pixel error too;
    of the pixels within six decades of the brightest, the median within
    1e-4 and at most 1 % off by more than 1e-3; the same sample counts, as
    the geodesic is the FP64 form's or follows it.  Fainter pixels are not
    bounded: as for the thermal fits, FP32 underflows where FP64 still
    resolves intensities many decades below the peak (most pixels of the
    log-polar image at 20 deg)."""
    from raptor_gb300 import engine
    d = torus64 if n == 64 else torus256
    gid = eng.upload_grid(d.geom, d.prims)
    desc = engine.image_desc(w, h, freqs, grid=gid, inclination=incl, camera=camera,
                             emission=engine.EMISSION_KAPPA)
    ref, sref = eng.render(desc, engine.PREC_FP64)
    st64 = eng.stats()
    img, spec = eng.render(desc, prec)
    st = eng.stats()
    assert st["rays"] == w * h and st["n_nonfinite"] == 0
    assert st["rt_samples"] == st64["rt_samples"]
    np.testing.assert_allclose(spec, sref, rtol=FLUX_RTOL_MIXED, atol=0)
    assert np.count_nonzero(ref) > 0.2 * ref.size
    nf = len(freqs)
    for f in range(nf):
        rf, gf = ref[f::nf], img[f::nf]
        l1 = float(np.sum(np.abs(gf - rf)) / np.sum(rf))
        bright = rf >= 1e-6 * rf.max()
        err = pixel_errors(gf[bright], rf[bright])
        info = (f, l1, float(np.median(err)), float(np.mean(err > 1e-3)), int(bright.sum()))
        assert l1 <= FLUX_RTOL_MIXED, info
        assert np.median(err) < 1e-4 and np.mean(err > 1e-3) <= 1e-2, info
    # a different image from the thermal model's
    thermal, _ = eng.render(engine.image_desc(w, h, freqs, grid=gid, inclination=incl, camera=camera), prec)
    assert not np.allclose(thermal, img, rtol=1e-3, atol=0.0)


@pytest.mark.parametrize("prec", [1, 2], ids=["mixed", "mixed_df"])
def test_kappa_adjoint_mixed_forms_match_fp64(torus64, prec):
    """The mixed forms' kappa adjoints (FP32 dual samples through the
    templated FP32 fits) against the FP64 kappa adjoint, whose gradients
    tests/test_gpu_vjp.py checks against central differences: the four
    scalars within 1e-4, each per-cell field within 1e-3 of its largest
    entry (the FP32 transfer's error, as for the thermal fits)."""
    from raptor_gb300 import engine
    eng = engine.Engine()
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    kw = dict(grid=gid, inclination=60.0, m_unit=1e19, r_high=3.0, r_low=3.0, emission=engine.EMISSION_KAPPA)
    mk = lambda **o: engine.image_desc(32, 32, [230e9, 345e9], **dict(kw, **o))  # noqa: E731
    target, _ = eng.render(mk(inclination=62.0, m_unit=1.3e19, r_high=4.0, r_low=4.0), engine.PREC_FP64)
    img64, _ = eng.render(mk(), engine.PREC_FP64)
    _, g64 = eng.vjp(mk(), img64 - target, engine.PREC_FP64)
    img, _ = eng.render(mk(), prec)
    _, g = eng.vjp(mk(), img - target, prec)
    eng.close()
    for key in ("d_m_unit", "d_r_high", "d_r_low", "d_inclination"):
        assert g[key] == pytest.approx(g64[key], rel=1e-4), key
    for key in ("d_rho", "d_u", "d_lnthetae"):
        scale = np.max(np.abs(g64[key]))
        assert scale > 0
        assert np.max(np.abs(g[key] - g64[key])) <= 1e-3 * scale, key
