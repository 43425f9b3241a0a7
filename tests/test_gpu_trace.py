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


@pytest.mark.parametrize("incl,pixel", [(60.0, 16 * 32 + 16), (17.0, 5 * 32 + 27)])
def test_trace_mixed_df_follows_fp64(torus64, incl, pixel):
    """The mixed-DF form's trace: the double-float geodesic follows the FP64
    one step for step (same step count, same transfer events, photon state
    within 1e-9 relative over the whole ray, where FP32 arithmetic would
    drift by ~1e-6); tau and I carry the FP32 transfer's error."""
    from raptor_gb300 import engine
    eng = engine.Engine()
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    d = engine.image_desc(32, 32, [230e9], grid=gid, inclination=incl)
    g64 = eng.trace_ray(d, pixel, engine.PREC_FP64)
    gdf = eng.trace_ray(d, pixel, engine.PREC_MIXED_DF)
    eng.close()
    assert len(gdf) == len(g64)
    scale = np.maximum(np.abs(g64[:, :9]), 1e-12)
    assert np.max(np.abs(gdf[:, :9] - g64[:, :9]) / scale) < 1e-9
    np.testing.assert_array_equal(gdf[:, 13], g64[:, 13])
    assert gdf[-1, 10] == pytest.approx(g64[-1, 10], rel=1e-4, abs=1e-300)
