"""The large differentiable configuration: five frequencies (86, 140, 230,
345 and 690 GHz) on the 512x512 torus.

* Reduced in rays (128x128 image), each form's VJP against central
  differences of the reference's own build rerun at perturbed parameters
  (tests/golden/vjp_fd_5freq_512.npz, made by tests/golden/make_vjp_fd.py
  --workload 5freq512): the four scalars and rho and u of 8 seeded cells, at the 1e-3
  bar of tests/test_gpu_vjp.py.
* At full size (2048x2048), the mixed form's forward render and VJP: every
  ray retired, the one-pass adjoint's own image within 1e-5 of the forward
  render's largest pixel, finite gradients, the Theta_e-field identity, and
  peak device memory within the workload's 60 GB budget (the adjoint keeps
  no checkpoints; the one pass's record tape holds 2048 records for each
  resident lane).
"""
import numpy as np
import pytest

from tests.parity import load_golden
from tests.test_gpu_vjp import Mismatches, _dln_thetae_unit_dR

pytestmark = pytest.mark.gpu

FREQS = [86e9, 140e9, 230e9, 345e9, 690e9]


@pytest.fixture(scope="module")
def torus512():
    from raptor_gb300 import synth
    return synth.make_torus(n1=512, n2=512, a=0.9375)


@pytest.mark.parametrize("prec", [1, 0, 2], ids=["mixed", "fp64", "mixed_df"])
def test_reduced_5freq_512_against_reference_finite_differences(torus512, prec):
    from raptor_gb300 import engine
    z = load_golden("vjp_fd_5freq_512.npz")
    w, h, n = (int(x) for x in z["image"])
    assert n == 512 and list(z["freqs"]) == FREQS
    eng = engine.Engine()
    try:
        gid = eng.upload_grid(torus512.geom, torus512.prims)
        desc = engine.image_desc(w, h, FREQS, grid=gid, inclination=60.0, m_unit=1e19, r_high=3.0, r_low=3.0)
        tdesc = engine.image_desc(w, h, FREQS, grid=gid, inclination=62.0, m_unit=1.3e19, r_high=4.0, r_low=4.0)
        target, _ = eng.render(tdesc, engine.PREC_FP64)
        img, _ = eng.render(desc, engine.PREC_FP64)
        dl = img - target
        assert 0.5 * np.sum(dl ** 2) == pytest.approx(z["L0"][0], rel=1e-6)
        _, g = eng.vjp(desc, dl, prec)
        assert eng.stats()["rays"] == w * h
    finally:
        eng.close()
    bad = Mismatches()
    bad.check("M_unit", g["d_m_unit"], z["rich_m_unit"][0])
    bad.check("R_high", g["d_r_high"], z["rich_r_high"][0])
    bad.check("R_low", g["d_r_low"], z["rich_r_low"][0])
    bad.check("inclination", g["d_inclination"], z["fd_incl_1e-07"][0])
    scale = max(np.max(np.abs(z["fd_rho"])), np.max(np.abs(z["fd_u"])))
    for k, (i, j) in enumerate(z["cells"]):
        bad.check_cell(f"rho[{i},{j}]", g["d_rho"][i, j], z["fd_rho"][k], scale)
        bad.check_cell(f"u[{i},{j}]", g["d_u"][i, j], z["fd_u"][k], scale)
    assert not bad, "\n".join(bad)


def test_full_size_2048_5freq_memory_and_identity(torus512):
    from raptor_gb300 import engine
    eng = engine.Engine()
    try:
        gid = eng.upload_grid(torus512.geom, torus512.prims)
        R = 3.0
        desc = engine.image_desc(2048, 2048, FREQS, grid=gid, inclination=60.0, m_unit=1e19, r_high=R, r_low=R)
        tdesc = engine.image_desc(2048, 2048, FREQS, grid=gid, inclination=62.0, m_unit=1.3e19, r_high=4.0,
                                  r_low=4.0)
        target, _ = eng.render(tdesc, engine.PREC_MIXED)
        img, spec = eng.render(desc, engine.PREC_MIXED)
        assert spec.shape == (5,) and np.all(spec > 0)
        fimg, g = eng.vjp(desc, img - target, engine.PREC_MIXED)
        st = eng.stats()
    finally:
        eng.close()
    assert float(np.abs(fimg - img).max()) <= 1e-5 * float(np.abs(img).max())
    assert st["device_ms"] == pytest.approx(st["kernel_ms"])  # one pass
    assert st["rays"] == 2048 * 2048 and st["n_nonfinite"] == 0
    assert st["peak_device_bytes"] <= 60e9, st["peak_device_bytes"]
    for k in ("d_m_unit", "d_r_high", "d_r_low", "d_inclination"):
        assert np.isfinite(g[k]) and g[k] != 0.0, k
    for k in ("d_rho", "d_u", "d_lnthetae"):
        assert np.all(np.isfinite(g[k])) and np.any(g[k] != 0.0), k
    total = float(np.sum(g["d_lnthetae"]))
    want = (g["d_r_high"] + g["d_r_low"]) / _dln_thetae_unit_dR(R)
    assert total == pytest.approx(want, rel=1e-4)
