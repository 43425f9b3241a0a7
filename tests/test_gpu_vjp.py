"""raptor_gpu_vjp against central finite differences: of the engine's own
FP64 forward render (small case), and of the reference build rerun at
perturbed parameters (tests/golden/vjp_fd_256.npz: 256x256 image of the
256x256 torus, loss to a target at M_unit x 1.3, R = 4, i = 62 deg).

Agreement bar: 1e-3 relative; a per-cell gradient to 1e-3 of its own
finite difference, or of 1e-3 of the largest per-cell difference where its
own is smaller than that.  M_unit, R_high and R_low are compared with
Richardson-extrapolated differences (4 D(h/2) - D(h)) / 3 at h = 1e-4
relative.  The image loss is only piecewise smooth in the inclination (clamps,
the min() of the step size and cell-index changes along 65,536 rays), so its
difference quotient at h = 1e-4 sits 0.7 % from the derivative on the 256x256
image and converges to it only as h shrinks (0.26 % at 1e-5, 2e-5 at 1e-6,
2e-8 at 1e-7 with the engine's own differences): the inclination gradient is
checked against the reference's difference at h = 1e-7, and the reference's
difference at h = 1e-4 is matched by the engine's own (a check of the forward
sensitivity, not of the VJP)."""
import numpy as np
import pytest

from tests.parity import load_golden

pytestmark = pytest.mark.gpu
TOL = 1e-3
REL_H = 1e-4


def _loss(eng, engine, desc, target):
    img, _ = eng.render(desc, engine.PREC_FP64)
    return 0.5 * float(np.sum((img - target) ** 2))


class Mismatches(list):
    def check(self, name, got, want, scale=None, tol=TOL):
        scale = abs(want) if scale is None else scale
        if not abs(got - want) <= tol * scale:
            self.append(f"{name}: vjp {got:.6e} vs finite difference {want:.6e}")

    def check_cell(self, name, got, want, largest, tol=TOL):
        """A per-cell gradient against its own difference quotient, floored
        at 1e-3 of the largest cell's (below that, the difference quotient of
        a 1e-4 perturbation is dominated by the loss's rounding and by the
        discrete decisions the perturbation flips)."""
        self.check(name, got, want, max(abs(want), 1e-3 * largest), tol)


@pytest.mark.parametrize("emission", [0, 1], ids=["thermal", "kappa"])
def test_vjp_against_engine_finite_differences(torus64, emission):
    """The FP64 VJP against central differences of the engine's FP64 render
    (the thermal fits, and the kappa fits, whose FP64 renders are pinned to
    the reference's kappa functions in tests/test_gpu_kappa.py)."""
    from raptor_gb300 import engine
    eng = engine.Engine()
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    kw = dict(grid=gid, inclination=60.0, m_unit=1e19, r_high=3.0, r_low=3.0, emission=emission)
    mk = lambda **o: engine.image_desc(32, 32, [230e9], **dict(kw, **o))  # noqa: E731
    target, _ = eng.render(mk(inclination=62.0, m_unit=1.3e19, r_high=4.0, r_low=4.0), engine.PREC_FP64)
    img, _ = eng.render(mk(), engine.PREC_FP64)
    _, g = eng.vjp(mk(), img - target, engine.PREC_FP64)
    bad = Mismatches()
    for key, attr in (("m_unit", "d_m_unit"), ("r_high", "d_r_high"), ("r_low", "d_r_low"),
                      ("inclination", "d_inclination")):
        d = []
        for rel in (REL_H, REL_H / 2):
            h = rel * kw[key]
            lp = _loss(eng, engine, mk(**{key: kw[key] + h}), target)
            lm = _loss(eng, engine, mk(**{key: kw[key] - h}), target)
            d.append((lp - lm) / (2 * h))
        fd = (4 * d[1] - d[0]) / 3
        if key == "inclination" and emission == engine.EMISSION_KAPPA:
            # the loss is only piecewise smooth in the inclination (module
            # docstring); on the kappa image the Richardson value at h = 1e-4
            # sits 1.6e-3 from the VJP, the plain differences at 1e-6 and 1e-7
            # within 1e-7 of it
            h = 1e-7 * kw[key]
            fd = (_loss(eng, engine, mk(**{key: kw[key] + h}), target) -
                  _loss(eng, engine, mk(**{key: kw[key] - h}), target)) / (2 * h)
        bad.check(key, g[attr], fd)
    # per-cell fields: cells in the torus body
    rng = np.random.default_rng(5)
    cand = np.argwhere(torus64.prims[0] > 0.3)
    cells = cand[rng.choice(len(cand), 6, replace=False)]
    fds, gots, names = [], [], []
    for (i, j) in cells:
        for q, field in ((0, "d_rho"), (1, "d_u")):
            pr = torus64.prims.copy()
            v = pr[q, i, j]
            pr[q, i, j] = v * (1 + REL_H)
            eng.upload_grid(torus64.geom, pr, grid_id=gid)
            lp = _loss(eng, engine, mk(), target)
            pr[q, i, j] = v * (1 - REL_H)
            eng.upload_grid(torus64.geom, pr, grid_id=gid)
            lm = _loss(eng, engine, mk(), target)
            fds.append((lp - lm) / (2 * REL_H * v))
            gots.append(g[field][i, j])
            names.append(f"{field}[{i},{j}]")
    eng.upload_grid(torus64.geom, torus64.prims, grid_id=gid)
    scale = max(abs(x) for x in fds)
    assert scale > 0
    for n, a, b in zip(names, gots, fds):
        bad.check_cell(n, a, b, scale)
    eng.close()
    assert not bad, "\n".join(bad)


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "mixed", "mixed_df"])
def test_vjp_against_reference_finite_differences(torus256, prec):
    """The reference rerun at perturbed parameters (the 256x256 adjoint workload), for
    each form's VJP: its one-pass adjoint (FP64; mixed: FP64 geodesic with
    FP32 tangents and the FP32 dual sample; mixed-DF: double-float geodesic,
    FP32 tangents and sample), all at the 1e-3 bar."""
    from raptor_gb300 import engine
    z = load_golden("vjp_fd_256.npz")
    eng = engine.Engine()
    gid = eng.upload_grid(torus256.geom, torus256.prims)
    desc = engine.image_desc(256, 256, [230e9], grid=gid, inclination=60.0, m_unit=1e19, r_high=3.0, r_low=3.0)
    tdesc = engine.image_desc(256, 256, [230e9], grid=gid, inclination=62.0, m_unit=1.3e19, r_high=4.0, r_low=4.0)
    target, _ = eng.render(tdesc, engine.PREC_FP64)
    img, _ = eng.render(desc, engine.PREC_FP64)
    dl = img - target
    assert 0.5 * np.sum(dl ** 2) == pytest.approx(z["L0"][0], rel=1e-6)
    fimg, g = eng.vjp(desc, dl, prec)
    # the one pass's own image: the adjoint's sums, rounded differently (FP64)
    assert np.abs(fimg - img).max() <= (1e-11 if prec == 0 else 1e-4) * np.abs(img).max()
    bad = Mismatches()
    bad.check("M_unit", g["d_m_unit"], z["rich_m_unit"][0])
    bad.check("R_high", g["d_r_high"], z["rich_r_high"][0])
    bad.check("R_low", g["d_r_low"], z["rich_r_low"][0])
    bad.check("inclination", g["d_inclination"], z["fd_incl_1e-07"][0])
    # the engine's own difference quotient at h = 1e-4 against the reference's
    h = 1e-4 * 60.0
    op, _ = eng.render(engine.image_desc(256, 256, [230e9], grid=gid, inclination=60.0 + h, m_unit=1e19,
                                         r_high=3.0, r_low=3.0), engine.PREC_FP64)
    om, _ = eng.render(engine.image_desc(256, 256, [230e9], grid=gid, inclination=60.0 - h, m_unit=1e19,
                                         r_high=3.0, r_low=3.0), engine.PREC_FP64)
    fd_engine = 0.5 * np.sum((op - om) * (op + om - 2 * target)) / (2 * h)
    if not abs(fd_engine - z["fd_incl"][0]) <= 1e-6 * abs(z["fd_incl"][0]):
        bad.append(f"inclination difference quotient at h=1e-4: engine {fd_engine:.9e} "
                   f"vs reference {z['fd_incl'][0]:.9e}")
    cells = z["cells"]
    scale = max(np.max(np.abs(z["fd_rho"])), np.max(np.abs(z["fd_u"])))
    for k, (i, j) in enumerate(cells):
        bad.check_cell(f"rho[{i},{j}]", g["d_rho"][i, j], z["fd_rho"][k], scale)
        bad.check_cell(f"u[{i},{j}]", g["d_u"][i, j], z["fd_u"][k], scale)
    assert eng.stats()["rays"] == 256 * 256
    eng.close()
    assert not bad, "\n".join(bad)


def _dln_thetae_unit_dR(R):
    """d ln Thetae_unit / d trat of raptor_harm_model.c:266-270 at trat = R."""
    tg = 0.5 * ((1.0 + 2.0 / 3.0 * (R + 1.0) / (R + 2.0)) + 4.0 / 3.0)
    return (1.0 / 3.0) / (R + 2.0) ** 2 / (tg - 1.0) - 1.0 / (1.0 + R)


def test_vjp_thetae_field_sums_to_temperature_ratio_gradient(torus64):
    """A uniform factor on Theta_e is a change of T_p/T_e when R_high = R_low
    (trat = R everywhere), and the bilinear weights of every sample sum to 1,
    so sum_cells dL/d ln f = (dL/dR_high + dL/dR_low) / (d ln Thetae_unit/dR)."""
    from raptor_gb300 import engine
    eng = engine.Engine()
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    R = 3.0
    desc = engine.image_desc(48, 48, [230e9, 345e9], grid=gid, inclination=60.0, m_unit=1e19, r_high=R, r_low=R)
    tdesc = engine.image_desc(48, 48, [230e9, 345e9], grid=gid, inclination=62.0, m_unit=1.3e19,
                              r_high=4.0, r_low=4.0)
    target, _ = eng.render(tdesc, engine.PREC_FP64)
    img, _ = eng.render(desc, engine.PREC_FP64)
    _, g = eng.vjp(desc, img - target, engine.PREC_FP64)
    eng.close()
    total = float(np.sum(g["d_lnthetae"]))
    want = (g["d_r_high"] + g["d_r_low"]) / _dln_thetae_unit_dR(R)
    assert want != 0.0
    assert total == pytest.approx(want, rel=1e-9)


@pytest.mark.parametrize("freqs", [[230e9], [86e9, 230e9, 345e9]])
def test_vjp_mixed(torus64, freqs):
    """precision = mixed: the mixed forward (FP64 geodesic, FP32 transfer)
    and its adjoint (the same FP64 path with FP32 inclination tangents, the
    FP32 dual sample).  Same steps and samples as the FP64 adjoint; gradients
    within 2e-3 of the FP64 adjoint's (scalars) and 2e-3 of scale (per-cell
    fields), the bar of the mixed-DF adjoint, which shares the sample; the
    Theta_e identity to FP32 accumulation accuracy."""
    from raptor_gb300 import engine
    eng = engine.Engine()
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    R = 3.0
    kw = dict(grid=gid, inclination=60.0, m_unit=1e19, r_high=R, r_low=R)
    desc = engine.image_desc(48, 48, freqs, **kw)
    tdesc = engine.image_desc(48, 48, freqs, **dict(kw, inclination=62.0, m_unit=1.3e19, r_high=4.0, r_low=4.0))
    target, _ = eng.render(tdesc, engine.PREC_FP64)
    img, _ = eng.render(desc, engine.PREC_FP64)
    dl = img - target
    i64, g64 = eng.vjp(desc, dl, engine.PREC_FP64)
    s64 = eng.stats()
    i32, g32 = eng.vjp(desc, dl, engine.PREC_MIXED)
    s32 = eng.stats()
    eng.close()
    assert np.abs(i64 - img).max() <= 1e-11 * np.abs(img).max()  # the FP64 one pass's own image
    assert np.abs(i32 - img).max() <= 1e-4 * np.abs(img).max()
    for key in ("rays", "steps", "rt_calls", "rt_samples"):
        assert s32[key] == s64[key], key
    for k in ("d_m_unit", "d_r_high", "d_r_low", "d_inclination"):
        assert g32[k] == pytest.approx(g64[k], rel=2e-3), k
    for k in ("d_rho", "d_u", "d_lnthetae"):
        scale = np.abs(g64[k]).max()
        assert scale > 0 and np.all(np.isfinite(g32[k]))
        assert np.abs(g32[k] - g64[k]).max() <= 2e-3 * scale, k
    total = float(np.sum(g32["d_lnthetae"]))
    want = (g32["d_r_high"] + g32["d_r_low"]) / _dln_thetae_unit_dR(R)
    assert total == pytest.approx(want, rel=1e-4)


@pytest.mark.parametrize("freqs", [[230e9], [86e9, 230e9, 345e9]])
def test_vjp_mixed_df(torus64, freqs):
    """precision = mixed-DF: the adjoint of the mixed-DF form (double-float
    geodesic and tangent, FP32 dual sample).  Its gradients agree with the
    FP64 adjoint's to 2e-3 (scalars) and 2e-3 of scale (per-cell fields):
    the two differentiate models whose images differ by the FP32 transfer's
    ~1e-6, and the DF adjoint accumulates in FP32.  The Theta_e identity
    holds to FP32 accumulation accuracy."""
    from raptor_gb300 import engine
    eng = engine.Engine()
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    R = 3.0
    kw = dict(grid=gid, inclination=60.0, m_unit=1e19, r_high=R, r_low=R)
    desc = engine.image_desc(48, 48, freqs, **kw)
    tdesc = engine.image_desc(48, 48, freqs, **dict(kw, inclination=62.0, m_unit=1.3e19, r_high=4.0, r_low=4.0))
    target, _ = eng.render(tdesc, engine.PREC_FP64)
    img, _ = eng.render(desc, engine.PREC_FP64)
    _, g64 = eng.vjp(desc, img - target, engine.PREC_FP64)
    idf, gdf = eng.vjp(desc, img - target, engine.PREC_MIXED_DF)
    st = eng.stats()
    eng.close()
    assert st["rays"] == 48 * 48
    assert np.abs(idf - img).max() <= 1e-4 * np.abs(img).max()
    for k in ("d_m_unit", "d_r_high", "d_r_low", "d_inclination"):
        assert gdf[k] == pytest.approx(g64[k], rel=2e-3), k
    for k in ("d_rho", "d_u", "d_lnthetae"):
        scale = np.abs(g64[k]).max()
        assert np.all(np.isfinite(gdf[k]))
        assert np.abs(gdf[k] - g64[k]).max() <= 2e-3 * scale, k
    total = float(np.sum(gdf["d_lnthetae"]))
    want = (gdf["d_r_high"] + gdf["d_r_low"]) / _dln_thetae_unit_dR(R)
    assert total == pytest.approx(want, rel=1e-4)


@pytest.mark.parametrize("camera,integrator", [(1, 4), (0, 2)])
def test_vjp_log_camera_and_rk2(torus64, camera, integrator):
    """The adjoint through the log-polar camera (its output factor enters
    dO/dI) and through RK2 steps: M_unit and inclination gradients against
    the engine's own central differences (h = 1e-6 relative, where the loss
    is smooth on this small image), and the mixed-DF and mixed adjoints
    against the FP64 one."""
    from raptor_gb300 import engine
    eng = engine.Engine()
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    kw = dict(grid=gid, inclination=55.0, m_unit=1e19, r_high=3.0, r_low=3.0, camera=camera,
              integrator=integrator)
    mk = lambda **o: engine.image_desc(24, 24, [230e9], **dict(kw, **o))  # noqa: E731
    target, _ = eng.render(mk(inclination=57.0, m_unit=1.2e19), engine.PREC_FP64)
    img, _ = eng.render(mk(), engine.PREC_FP64)
    _, g = eng.vjp(mk(), img - target, engine.PREC_FP64)
    _, gdf = eng.vjp(mk(), img - target, engine.PREC_MIXED_DF)
    _, gmx = eng.vjp(mk(), img - target, engine.PREC_MIXED)
    bad = Mismatches()
    for key, attr in (("m_unit", "d_m_unit"), ("inclination", "d_inclination")):
        h = 1e-6 * kw[key]
        lp = _loss(eng, engine, mk(**{key: kw[key] + h}), target)
        lm = _loss(eng, engine, mk(**{key: kw[key] - h}), target)
        bad.check(key, g[attr], (lp - lm) / (2 * h))
        bad.check(key + " (mixed-DF)", gdf[attr], g[attr])
        bad.check(key + " (mixed)", gmx[attr], g[attr])
    eng.close()
    assert not bad, "\n".join(bad)


@pytest.mark.parametrize("camera,integrator,freqs", [(0, 4, [230e9]), (1, 2, [230e9]),
                                                     (0, 4, [86e9, 230e9, 345e9])])
def test_vjp_sample_pool_matches_in_place(torus256, camera, integrator, freqs):
    """The FP64 adjoint with the per-warp sample pool (vjp_kernel_pool; with
    several frequencies its results go through the scratch buffer) against
    the in-place kernel (no_sample_pool), both in two passes: the same step,
    sample and term counts, scalar gradients within 1e-12 and per-cell
    gradients within 1e-12 of the largest (the FP64 atomics of the per-cell
    scatter add in a different order)."""
    from raptor_gb300 import engine
    out = {}
    for nsp in (0, 1):
        eng = engine.Engine(no_sample_pool=nsp, vjp_tape=-1)
        gid = eng.upload_grid(torus256.geom, torus256.prims)
        mk = lambda **o: engine.image_desc(64, 64, freqs, **dict(dict(grid=gid, inclination=60.0, camera=camera, integrator=integrator), **o))  # noqa: E731
        target, _ = eng.render(mk(inclination=62.0, m_unit=1.3e19, r_high=4.0, r_low=4.0), engine.PREC_FP64)
        img, _ = eng.render(mk(), engine.PREC_FP64)
        _, g = eng.vjp(mk(), img - target, engine.PREC_FP64)
        out[nsp] = (g, eng.stats())
        eng.close()
    (g0, s0), (g1, s1) = out[0], out[1]
    for key in ("steps", "rt_samples", "vjp_terms", "vjp_gated_terms", "rays"):
        assert s0[key] == s1[key], key
    for key in ("d_m_unit", "d_r_high", "d_r_low", "d_inclination"):
        assert g0[key] == pytest.approx(g1[key], rel=1e-12, abs=0.0), key
    for key in ("d_rho", "d_u", "d_lnthetae"):
        scale = float(np.abs(g1[key]).max())
        assert scale > 0.0 and float(np.abs(g0[key] - g1[key]).max()) <= 1e-12 * scale, key


@pytest.mark.parametrize("prec", [0, 1, 2], ids=["fp64", "mixed", "mixed_df"])
def test_vjp_ranges_add_up(torus64, prec):
    """raptor_gpu_vjp_range: the gradients of disjoint ray ranges add up to
    the whole image's (every gradient is a sum over rays; the per-cell
    atomics add in another order), and the partial images to the whole
    image - the split raptor_gb300/shard.py makes across processes."""
    from raptor_gb300 import engine
    eng = engine.Engine()
    gid = eng.upload_grid(torus64.geom, torus64.prims)
    desc = engine.image_desc(30, 26, [86e9, 230e9], grid=gid, inclination=55.0)
    target, _ = eng.render(engine.image_desc(30, 26, [86e9, 230e9], grid=gid, inclination=57.0, m_unit=1.2e19),
                           engine.PREC_FP64)
    img, _ = eng.render(desc, engine.PREC_FP64)
    dl = img - target
    full_img, full = eng.vjp(desc, dl, prec)
    cuts = [0, 97, 401, 30 * 26]
    parts = [eng.vjp(desc, dl, prec, ray_begin=a, ray_count=b - a) for a, b in zip(cuts, cuts[1:])]
    assert eng.stats()["rays"] == cuts[-1] - cuts[-2]
    eng.close()
    np.testing.assert_allclose(sum(p[0] for p in parts), full_img, rtol=1e-12, atol=0)
    for k in ("d_m_unit", "d_r_high", "d_r_low", "d_inclination"):
        assert sum(p[1][k] for p in parts) == pytest.approx(full[k], rel=1e-9), k
    for k in ("d_rho", "d_u", "d_lnthetae"):
        scale = float(np.abs(full[k]).max())
        assert float(np.abs(sum(p[1][k] for p in parts) - full[k]).max()) <= 1e-9 * scale, k
