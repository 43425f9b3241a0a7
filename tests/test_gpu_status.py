"""Status codes of a finished render.

Rays that end with a non-finite photon state or intensity make the render
an error (RAPTOR_ERR_NONFINITE) with the outputs still written; rays stopped
by the step cap - which the reference applies without notice - a warning
(RAPTOR_WARN_STEPCAP) with the image complete.  Both come from real inputs:
a camera at inclination exactly 0 (the reference's initialize_photon forms
0 * inf there, metric.c:662-668, and renders an empty image) and a step
size small enough that every ray needs more than max_steps = 1e5 steps
(parameters.h:182).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from raptor_gb300 import engine
    e = engine.Engine()
    yield e
    e.close()


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "mixed", "mixed_df"])
def test_face_on_camera_is_nonfinite(eng, torus64, prec):
    from oracle import port
    from raptor_gb300 import engine
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    desc = engine.image_desc(6, 5, [230e9], grid=gid, inclination=0.0)
    out = np.full(30, -1.0)
    spec = np.full(1, -1.0)
    rc = eng.lib.raptor_gpu_render(eng.h, ctypes.byref(desc), 1, prec, engine._dp(out), engine._dp(spec))
    assert rc == engine.ERR_NONFINITE, rc
    assert "non-finite" in eng.lib.raptor_gpu_last_error(eng.h).decode()
    st = eng.stats()
    assert st["rays"] == 30 and st["n_nonfinite"] == 30
    # the outputs are written, as the reference writes them: an empty image
    ref, _ = port.Scene(torus64.geom, torus64.prims, 6, 5, inclination=0.0).render([230e9])
    assert np.array_equal(out, ref[:, 0]) and not np.any(out) and spec[0] == 0.0
    with pytest.raises(engine.EngineError) as e:
        eng.render(desc, prec)
    assert e.value.code == engine.ERR_NONFINITE
    # a normal render afterwards is unaffected
    eng.render(engine.image_desc(6, 5, [230e9], grid=gid, inclination=60.0), prec)
    assert eng.last_status == 0


@pytest.mark.parametrize("prec", [0, 2], ids=["fp64", "mixed_df"])
def test_step_cap_is_a_warning(eng, torus64, prec):
    from raptor_gb300 import engine
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    desc = engine.image_desc(2, 2, [230e9], grid=gid, inclination=60.0, stepsize=5e-5, cam_size_x=8.0,
                             cam_size_y=8.0)
    with pytest.warns(engine.EngineWarning, match="step cap"):
        img, spec = eng.render(desc, prec)
    assert eng.last_status == engine.WARN_STEPCAP
    st = eng.stats()
    assert st["rays"] == 4 and st["n_stepcap"] == 4 and st["max_ray_steps"] == 100000
    assert st["n_nonfinite"] == 0 and np.all(np.isfinite(img)) and np.isfinite(spec[0])
