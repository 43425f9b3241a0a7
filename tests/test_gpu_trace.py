"""Step-by-step agreement of one ray between the engine and the oracle
(raptor_gpu_trace_ray vs port_trace_ray)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("incl,pixel,eps", [(60.0, 16 * 32 + 16, 0.05), (17.0, 5 * 32 + 27, 0.05),
                                             (35.0, 100, 0.1)])
def test_trace_matches_port(torus64, incl, pixel, eps):
    from oracle import port
    from raptor_gb300 import engine
    eng = engine.Engine()
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    d = engine.image_desc(32, 32, [230e9], grid=gid, inclination=incl, stepsize=eps)
    g = eng.trace_ray(d, pixel, engine.PREC_FP64)
    eng.close()
    p = port.Scene(torus64.geom, torus64.prims, 32, 32, inclination=incl, stepsize=eps).trace_ray(pixel, [230e9])
    assert abs(len(g) - len(p)) <= 1
    n = min(len(g), len(p), 40)
    # photon state and step size agree to rounding over the first steps
    scale = np.maximum(np.abs(p[:n, :9]), 1e-12)
    assert np.max(np.abs(g[:n, :9] - p[:n, :9]) / scale) < 1e-9
    np.testing.assert_array_equal(g[:n, 13], p[:n, 13])  # same transfer events
    # final intensity of the first frequency
    assert g[-1, 10] == pytest.approx(p[-1, 10], rel=1e-6, abs=1e-300)
