"""The oracle (C port) pinned against the reference's own outputs: golden
fixtures made by tests/golden/make_golden.py from the reference build."""
import os

import numpy as np
import pytest

from tests.parity import assert_fp64_parity, load_golden


@pytest.fixture(scope="module")
def small():
    return load_golden("small_g64.npz")


def _scene(dump, params):
    from oracle import port
    w, h, incl, freq, rk, eps, mu, rh, rl = params
    return port.Scene(dump.geom, dump.prims, int(w), int(h), inclination=incl, stepsize=eps, m_unit=mu,
                      r_high=rh, r_low=rl, integrator=int(rk)), freq


def test_generator_matches_golden(torus64, small):
    from tests.golden.make_golden import prim_checksum
    np.testing.assert_allclose(prim_checksum(torus64.prims), small["prim_checksum"], rtol=1e-12)


@pytest.mark.parametrize("name", ["g64_i60_rk4", "g64_i17_rk4", "g64_i120_rk4_86", "g64_i60_rk2",
                                  "g64_i35_rk4_odd"])
def test_port_matches_reference_images(torus64, small, name):
    sc, freq = _scene(torus64, small[f"{name}_params"])
    out, _ = sc.render([freq])
    assert_fp64_parity(out[:, 0], small[f"{name}_img"], name)
    np.testing.assert_allclose(out[:, 0].sum(), small[f"{name}_spec"][0], rtol=1e-6)


def test_port_matches_reference_100x100_on_256(torus256):
    g = load_golden("img100_g256.npz")
    from tests.golden.make_golden import prim_checksum
    np.testing.assert_allclose(prim_checksum(torus256.prims), g["prim_checksum"], rtol=1e-12)
    sc, freq = _scene(torus256, g["params"])
    out, _ = sc.render([freq])
    assert_fp64_parity(out[:, 0], g["img"], "100x100 on 256^2")


def test_port_function_kats(torus64, small):
    sc, _ = _scene(torus64, small["g64_i60_rk4_params"])
    for k, X in enumerate(small["kat_X"]):
        np.testing.assert_allclose(sc.metric_dd(X).ravel(), small["kat_gdd"][k], rtol=1e-13, atol=1e-300)
        np.testing.assert_allclose(sc.metric_uu(X).ravel(), small["kat_guu"][k], rtol=1e-13, atol=1e-300)
        np.testing.assert_allclose(sc.connection(X).ravel(), small["kat_gamma"][k], rtol=1e-12, atol=1e-14)
    from oracle import port
    lib = port.load()
    lat = small["kat_lattice"]
    for i, (B, cp, th, nu, ne) in enumerate(lat):
        j = lib.port_j_thsynch(B, cp, th, nu, ne)
        # exp(-X^(1/3)) with X^(1/3) up to ~600 amplifies argument rounding
        assert j == pytest.approx(small["kat_j"][i], rel=1e-11, abs=0)
        assert lib.port_a_th(j, nu, th) == pytest.approx(small["kat_a"][i], rel=1e-11, abs=0)
    for k, X in enumerate(small["kat_fluid_X"]):
        ok, f = sc.fluid(X)
        assert ok == small["kat_fluid_ok"][k]
        # u^1 = V^1 - Vfac g^{01} cancels; compare to 1e-11 relative or 1e-15 absolute
        np.testing.assert_allclose(f, small["kat_fluid"][k], rtol=1e-11, atol=1e-15)


def test_connection_is_metric_derivative(torus64, small):
    """Gamma^i_jk = 1/2 g^il (d_j g_lk + d_k g_lj - d_l g_jk) by central
    differences (the reference's connection_num_udd check, metric.c:255-328)."""
    sc, _ = _scene(torus64, small["g64_i60_rk4_params"])
    h = 1e-6
    for X in small["kat_X"][:8]:
        dg = np.zeros((4, 4, 4))
        for l in (1, 2):
            Xp = X.copy(); Xp[l] += h
            Xm = X.copy(); Xm[l] -= h
            dg[l] = (sc.metric_dd(Xp) - sc.metric_dd(Xm)) / (2 * h)
        gi = sc.metric_uu(X)
        G = 0.5 * (np.einsum("il,jlk->ijk", gi, dg) + np.einsum("il,klj->ijk", gi, dg)
                   - np.einsum("il,ljk->ijk", gi, dg))
        np.testing.assert_allclose(sc.connection(X), G, rtol=2e-5, atol=1e-7 * np.abs(G).max())


def test_initial_photon_is_null(torus64, small):
    sc, _ = _scene(torus64, small["g64_i60_rk4_params"])
    for alpha, beta in [(-7.3, 3.1), (0.4, -12.0), (19.0, 19.0), (-0.2, 0.2)]:
        ph = sc.init_photon(alpha, beta)
        g = sc.metric_dd(ph[:4])
        kk = ph[4:] @ g @ ph[4:]
        assert abs(kk) / ph[4] ** 2 < 1e-9


def test_camera_angle_root(torus64, small):
    sc, _ = _scene(torus64, small["g64_i60_rk4_params"])
    x2 = sc.camera_x2()
    th = np.pi * x2 + 0.5 * (1 - 0.3) * np.sin(2 * np.pi * x2)
    assert th == pytest.approx(np.arccos(np.cos(np.radians(60.0))), abs=1e-14)


def _reference_sources():
    from oracle import ref
    return ref.sources_present()


@pytest.mark.skipif(not _reference_sources(), reason="reference sources not present on this machine")
def test_port_vs_reference_fresh_seed(tmp_path):
    """Port against the reference build on a torus the fixtures never saw."""
    from oracle import port, ref
    from raptor_gb300 import harm, synth
    from tests.golden.make_golden import quiet
    d = synth.make_torus(n1=64, n2=64, a=0.5, seed=99)
    path = str(tmp_path / "t.dump")
    harm.write_dump(path, d)
    model = harm.ModelIn(IMG_WIDTH=20, IMG_HEIGHT=20, STEPSIZE=0.05)
    with quiet():
        s = ref.RefSession(path, model, 2e19, 75.0, 5.0, 2.0, 0.0, n1=64, n2=64, workdir=str(tmp_path))
        img, spec, _ = s.render_serial(345e9)
    sc = port.Scene(d.geom, d.prims, 20, 20, inclination=75.0, m_unit=2e19, r_high=5.0, r_low=2.0)
    out, _ = sc.render([345e9])
    assert_fp64_parity(out[:, 0], img, "fresh seed")


@pytest.mark.parametrize("name", ["log_i60_rk4", "log_i17_rk2"])
def test_port_matches_reference_log_camera(torus256, name):
    """LOG_IMPACT_CAM build of the reference (parameters.h:54-55): log-polar
    impact parameters (integrator.c:192-198) and the r dr dtheta / D^2
    post-scale of calculate_image (core.c:123-133)."""
    from oracle import port
    g = load_golden("logcam_g256.npz")
    from tests.golden.make_golden import prim_checksum
    np.testing.assert_allclose(prim_checksum(torus256.prims), g["prim_checksum"], rtol=1e-12)
    w, h, incl, freq, rk = g[f"{name}_params"]
    sc = port.Scene(torus256.geom, torus256.prims, int(w), int(h), inclination=incl, integrator=int(rk), camera=1)
    out, _ = sc.render([freq])
    assert_fp64_parity(out[:, 0], g[f"{name}_img"], name)
    np.testing.assert_allclose(out[:, 0].sum(), g[f"{name}_spec"][0], rtol=1e-6)


@pytest.mark.parametrize("k,name", [(0, "a05_i120_345"), (1, "a09375_i25_86")])
def test_port_matches_reference_batch_dumps(k, name):
    """The two dumps of the batched configuration (a = 0.5 and a = 0.9375 with
    their own seeds): one image each, M_unit 3e18 (optically thin) and 5e19
    (optically thick at 86 GHz)."""
    from oracle import port
    from raptor_gb300 import workloads
    from tests.golden.make_golden import prim_checksum
    g = load_golden("batch_dumps_g256.npz")
    d = workloads.batch_dumps(256)[k]
    np.testing.assert_allclose(prim_checksum(d.prims), g[f"{name}_prim_checksum"], rtol=1e-12)
    sc, freq = _scene(d, g[f"{name}_params"])
    out, _ = sc.render([freq])
    assert_fp64_parity(out[:, 0], g[f"{name}_img"], name)
    np.testing.assert_allclose(out[:, 0].sum(), g[f"{name}_spec"][0], rtol=1e-6)


@pytest.mark.parametrize("name", ["r0_i50_rk4", "r0_i130_rk2"])
def test_port_matches_reference_nonzero_r0(name):
    """A non-zero MKS radial offset (R0 = 0.3 in the dump header): r = R0 +
    exp(x1) in the metric and connection (metric.c:94-137, 538-638)."""
    from tests.golden.make_golden import prim_checksum, r0_dump
    g = load_golden("r0_g64.npz")
    d = r0_dump()
    assert d.geom.R0 == g["R0"][0]
    np.testing.assert_allclose(prim_checksum(d.prims), g["prim_checksum"], rtol=1e-12)
    sc, freq = _scene(d, g[f"{name}_params"])
    out, _ = sc.render([freq])
    assert_fp64_parity(out[:, 0], g[f"{name}_img"], name)


# ---- kappa-distribution emission (j_nu.c:28-106) ----

def _kappa_hyp_params():
    k = 3.5
    a, b, c = k - 1 / 3, k + 1, k + 2 / 3
    return a, b, c


def test_port_hyp2f1_against_scipy():
    """The oracle's Gauss hypergeometric function (in place of GSL's, which
    is absent) against scipy's hyp2f1 on every argument range the kappa
    absorptivity reaches: 2F1(a, b; c; z) for z in [-1, 0), and the
    connection formula's two functions at w = 1/(1 - z) in (0, 1/2)."""
    special = pytest.importorskip("scipy.special")
    from oracle import port
    lib = port.load()
    a, b, c = _kappa_hyp_params()
    worst = 0.0
    for z in -np.geomspace(1e-6, 1.0, 300):
        worst = max(worst, abs(lib.port_hyp2f1(a, b, c, z) / special.hyp2f1(a, b, c, z) - 1))
    for w in np.linspace(1e-6, 0.5, 300):
        for p, q, r in ((a, c - b, a - b + 1), (b, c - a, b - a + 1)):
            worst = max(worst, abs(lib.port_hyp2f1(p, q, r, w) / special.hyp2f1(p, q, r, w) - 1))
    assert worst < 1e-13, worst


def test_kappa_series_tables():
    """csrc/kappa_tables.inc (written by csrc/gen_kappa_tables.py) holds the
    exact power-series coefficients rounded to double, and 80 terms sum the
    two series to scipy's hyp2f1 within 1e-14 on [0, 1/2]."""
    import importlib.util
    import re
    special = pytest.importorskip("scipy.special")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("gkt", os.path.join(root, "raptor_gb300", "csrc",
                                                                      "gen_kappa_tables.py"))
    gkt = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gkt)
    src = open(os.path.join(root, "raptor_gb300", "csrc", "kappa_tables.inc")).read()
    for name, p, q, r, _ in gkt.series():
        m = re.search(name + r"\[(\d+)\] = \{(.*?)\};", src, re.S)
        assert m, name
        vals = [float(t) for t in m.group(2).replace("\n", " ").split(",") if t.strip()]
        assert len(vals) == int(m.group(1)) == gkt.N_TERMS
        assert vals == [float(v) for v in gkt.coefficients(p, q, r)], name
        for x in np.linspace(0.0, 0.5, 101):
            s = 0.0
            for v in reversed(vals):
                s = s * x + v
            assert abs(s / special.hyp2f1(float(p), float(q), float(r), x) - 1) < 1e-14, (name, x)


def test_port_kappa_matches_reference_functions():
    """The port's kappa emissivity and absorptivity against the reference's
    own emission_coeff_kappa_FIT / absorption_coeff_kappa_FIT (built from its
    sources with the oracle's 2F1 in GSL's place) on seeded plasma states."""
    import ctypes
    from oracle import port, ref
    if not ref.available(64, 64):
        pytest.skip("the reference's sources are not staged on this machine")
    lib = ref.load(64, 64, "RK4")
    lib.ref_kappa_coeffs.argtypes = [ctypes.c_double] * 5 + [ctypes.POINTER(ctypes.c_double)]
    pl = port.load()
    out = (ctypes.c_double * 2)()
    rng = np.random.default_rng(35)
    n_nonzero = 0
    for _ in range(3000):
        nu, ne = 10 ** rng.uniform(9, 13), 10 ** rng.uniform(2, 8)
        th, B, cth = 10 ** rng.uniform(-2.5, 3), 10 ** rng.uniform(-2, 3), rng.uniform(-0.999, 0.999)
        lib.ref_kappa_coeffs(nu, ne, th, B, cth, out)
        got = (pl.port_j_kappa(nu, ne, th, B, cth), pl.port_a_kappa(nu, ne, th, B, cth))
        for g, w in zip(got, out):
            assert g == pytest.approx(w, rel=1e-13, abs=0.0)
            n_nonzero += w != 0.0
    # the special cases: the nu_p sentinel, a clamped pitch angle, |z| = 1
    for args in ((1.0, 1e5, 10.0, 20.0, 0.3), (2e11, 1e5, 10.0, 20.0, 1.0), (2e11, 1e5, 1 / 3.5, 20.0, 0.3)):
        lib.ref_kappa_coeffs(*args, out)
        assert (pl.port_j_kappa(*args), pl.port_a_kappa(*args)) == (out[0], out[1])
    assert n_nonzero > 5000
