"""The kappa-distribution emission model (RAPTOR_EMISSION_KAPPA): the fits of
j_nu.c:28-106, kappa = 3.5, in place of the thermal ones, rendered by the
FP64 form and compared with the oracle port, whose kappa functions equal
the reference's own (tests/test_oracle.py), at the FP64 parity bar of
tests/parity.py.  The mixed forms, the adjoint and the mixed traces refuse
kappa images with RAPTOR_ERR_INVALID."""
import numpy as np
import pytest

from tests.parity import assert_fp64_parity

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


def test_kappa_refused_outside_fp64(eng, torus64):
    from raptor_gb300 import engine
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    desc = engine.image_desc(8, 8, [230e9], grid=gid, emission=engine.EMISSION_KAPPA)
    for prec in (engine.PREC_MIXED, engine.PREC_MIXED_DF):
        with pytest.raises(engine.EngineError) as e:
            eng.render(desc, prec)
        assert e.value.code == -1
    img, _ = eng.render(desc, engine.PREC_FP64)
    with pytest.raises(engine.EngineError) as e:
        eng.vjp(desc, img, engine.PREC_FP64)
    assert e.value.code == -1
    with pytest.raises(engine.EngineError):
        eng.render(engine.image_desc(8, 8, [230e9], grid=gid, emission=2))
    # the context stays usable
    eng.render(desc, engine.PREC_FP64)
