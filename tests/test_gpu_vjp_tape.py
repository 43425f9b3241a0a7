"""The one-pass adjoint (raptor_gpu_vjp's default: the pooled FP64 adjoint,
the mixed and the mixed-DF ones) against the two-pass VJP
(options.vjp_tape = -1: the forward render, then the adjoint reading each
pixel's I from it).

The one pass keeps each ray's per-cell terms on a per-lane tape and closes
them with the ray's own I when the ray ends.  The scalar gradients do not
involve I: equal to 1e-12 (the order of the per-warp atomics).  The
per-cell gradients take the suffix of I from the ray's own sums instead of
the forward image, which differ by the transfer's rounding: within 1e-4 of
the largest cell's for the FP32 transfers, 1e-9 in FP64.  The image the
call returns is the pass's own: within 1e-5 of the forward render's
largest pixel (1e-11 in FP64), and each bright pixel (above 1e-3 of the
largest) within 1e-4 of its own value (1e-10 in FP64).
A tape too short for some ray makes the call fall back to two passes: the
two-pass gradients and image.  The finite-difference tests of
tests/test_gpu_vjp.py and tests/test_gpu_vjp_5freq_512.py run the one
pass, the default."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCALARS = ("d_m_unit", "d_r_high", "d_r_low", "d_inclination")
FIELDS = ("d_rho", "d_u", "d_lnthetae")


def _vjp(torus, opts, desc_kw, tgt_kw, freqs, prec, want_fields=True):
    from raptor_gb300 import engine
    eng = engine.Engine(**opts)
    gid = eng.upload_grid(torus.geom, torus.prims)
    desc = engine.image_desc(40, 36, freqs, grid=gid, **desc_kw)
    target, _ = eng.render(engine.image_desc(40, 36, freqs, grid=gid, **tgt_kw), engine.PREC_FP64)
    fwd, _ = eng.render(desc, prec)
    img, g = eng.vjp(desc, fwd - target, prec, want_fields=want_fields)
    st = eng.stats()
    eng.close()
    return fwd, img, g, st


CASES = [
    (1, [230e9], 0), (1, [86e9, 230e9, 345e9], 0), (2, [230e9], 0), (2, [86e9, 230e9, 345e9], 0),
    (1, [230e9, 345e9], 1), (2, [230e9, 345e9], 1), (0, [230e9], 0), (0, [86e9, 230e9, 345e9], 0),
    (0, [230e9, 345e9], 1),
]
# (image vs the largest pixel, bright pixels, per-cell fields vs the largest)
BARS = {0: (1e-11, 1e-10, 1e-9), 1: (1e-5, 1e-4, 1e-4), 2: (1e-5, 1e-4, 1e-4)}


@pytest.mark.parametrize("prec,freqs,emission", CASES,
                         ids=["mixed-1f", "mixed-3f", "mixed_df-1f", "mixed_df-3f", "mixed-kappa", "mixed_df-kappa",
                              "fp64-1f", "fp64-3f", "fp64-kappa"])
def test_one_pass_matches_two_passes(torus64, prec, freqs, emission):
    bar_img, bar_bright, bar_field = BARS[prec]
    kw = dict(inclination=60.0, m_unit=1e19, r_high=3.0, r_low=3.0, emission=emission)
    tkw = dict(kw, inclination=62.0, m_unit=1.3e19, r_high=4.0, r_low=4.0)
    fwd, img1, g1, s1 = _vjp(torus64, {}, kw, tkw, freqs, prec)
    _, img2, g2, s2 = _vjp(torus64, {"vjp_tape": -1}, kw, tkw, freqs, prec)
    # two passes return the forward render; one pass its own image
    assert np.array_equal(img2, fwd)
    peak = float(np.abs(fwd).max())
    assert peak > 0 and float(np.abs(img1 - fwd).max()) <= bar_img * peak
    bright = np.abs(fwd) > 1e-3 * peak
    assert float(np.max(np.abs(img1[bright] - fwd[bright]) / np.abs(fwd[bright]))) <= bar_bright
    # the same rays, steps and samples; the one pass has no forward render
    for key in ("rays", "steps", "rt_calls", "rt_samples", "vjp_terms", "vjp_gated_terms", "n_nonfinite",
                "n_stepcap"):
        assert s1[key] == s2[key], key
    assert s1["device_ms"] == pytest.approx(s1["kernel_ms"])
    for k in SCALARS:
        assert g1[k] == pytest.approx(g2[k], rel=1e-12, abs=0.0), k
    for k in FIELDS:
        scale = float(np.abs(g2[k]).max())
        assert scale > 0 and np.all(np.isfinite(g1[k]))
        assert float(np.abs(g1[k] - g2[k]).max()) <= bar_field * scale, k


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "mixed", "mixed_df"])
def test_tape_full_falls_back_to_two_passes(torus64, prec):
    """Two records per lane: rays with more samples inside the gate fill the
    tape, and the call reruns as two passes."""
    kw = dict(inclination=60.0, m_unit=1e19, r_high=3.0, r_low=3.0)
    tkw = dict(kw, inclination=62.0, m_unit=1.3e19)
    freqs = [86e9, 230e9]
    fwd, img1, g1, s1 = _vjp(torus64, {"vjp_tape": 2}, kw, tkw, freqs, prec)
    _, img2, g2, s2 = _vjp(torus64, {"vjp_tape": -1}, kw, tkw, freqs, prec)
    assert np.array_equal(img1, fwd) and np.array_equal(img2, fwd)
    assert s1["device_ms"] > s1["kernel_ms"]  # a forward render ran
    for k in SCALARS:
        assert g1[k] == pytest.approx(g2[k], rel=1e-12, abs=0.0), k
    for k in FIELDS:
        scale = float(np.abs(g2[k]).max())
        assert scale > 0 and float(np.abs(g1[k] - g2[k]).max()) <= 1e-12 * scale, k


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "mixed", "mixed_df"])
def test_one_pass_scalars_without_fields(torus64, prec):
    """Without the per-cell fields the one pass writes no records: the same
    scalar gradients and image."""
    kw = dict(inclination=50.0, m_unit=1e19, r_high=3.0, r_low=3.0)
    tkw = dict(kw, inclination=52.0, r_high=4.0)
    freqs = [230e9]
    _, img1, g1, _ = _vjp(torus64, {}, kw, tkw, freqs, prec, want_fields=False)
    _, img2, g2, _ = _vjp(torus64, {}, kw, tkw, freqs, prec, want_fields=True)
    assert np.array_equal(img1, img2)
    for k in SCALARS:
        assert g1[k] == pytest.approx(g2[k], rel=1e-12, abs=0.0), k
