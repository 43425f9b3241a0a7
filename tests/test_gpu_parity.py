"""Parity of the CUDA engine (through its C ABI) with the reference's
outputs (golden fixtures) and with the oracle port.

FP64 form: per-pixel relative error <= 1e-6 except <= 0.1% grazing pixels,
total flux within 1e-6 (tests/parity.py).  Mixed form: total flux within 1e-4.
"""
import numpy as np
import pytest

from tests.parity import FLUX_RTOL_MIXED, assert_fp64_parity, load_golden, pixel_errors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from raptor_gb300 import engine
    e = engine.Engine()
    yield e
    e.close()


def _grid(eng, dump):
    """Upload each dump once per engine (the context holds 16 grid slots).
    The cache holds the dump itself, so its id cannot be reused by another."""
    cache = eng.__dict__.setdefault("_test_grids", {})
    if id(dump) not in cache:
        cache[id(dump)] = (dump, eng.upload_grid(dump.geom, dump.prims))
    return cache[id(dump)][1]


@pytest.fixture(scope="module")
def small():
    return load_golden("small_g64.npz")


def _desc(params, grid):
    from raptor_gb300 import engine
    w, h, incl, freq, rk, eps, mu, rh, rl = params
    return engine.image_desc(int(w), int(h), [freq], grid=grid, inclination=incl, stepsize=eps, m_unit=mu,
                             r_high=rh, r_low=rl, integrator=int(rk))


NAMES = ["g64_i60_rk4", "g64_i17_rk4", "g64_i120_rk4_86", "g64_i60_rk2", "g64_i35_rk4_odd"]


@pytest.mark.parametrize("name", NAMES)
def test_fp64_matches_reference_small(eng, torus64, small, name):
    from raptor_gb300 import engine
    gid = _grid(eng, torus64)
    img, spec = eng.render(_desc(small[f"{name}_params"], gid), engine.PREC_FP64)
    assert_fp64_parity(img, small[f"{name}_img"], name)
    assert spec[0] == pytest.approx(small[f"{name}_spec"][0], rel=1e-6)
    st = eng.stats()
    assert st["rays"] == img.size and st["n_nonfinite"] == 0


def test_fp64_matches_reference_100x100_on_256(eng, torus256):
    from raptor_gb300 import engine
    g = load_golden("img100_g256.npz")
    gid = _grid(eng, torus256)
    img, spec = eng.render(_desc(g["params"], gid), engine.PREC_FP64)
    assert_fp64_parity(img, g["img"], "100x100 on 256^2")
    assert spec[0] == pytest.approx(g["spec"][0], rel=1e-6)


@pytest.mark.parametrize("name", ["log_i60_rk4", "log_i17_rk2"])
def test_log_camera_matches_reference(eng, torus256, name):
    """LOG_IMPACT_CAM: log-polar impact parameters and the r dr dtheta / D^2
    output scale; FP64 at the parity bar, mixed form within its flux bar."""
    from raptor_gb300 import engine
    g = load_golden("logcam_g256.npz")
    w, h, incl, freq, rk = g[f"{name}_params"]
    d = engine.image_desc(int(w), int(h), [freq], grid=_grid(eng, torus256), inclination=incl,
                          integrator=int(rk), camera=engine.CAM_LOG)
    img, spec = eng.render(d, engine.PREC_FP64)
    assert_fp64_parity(img, g[f"{name}_img"], name)
    assert spec[0] == pytest.approx(g[f"{name}_spec"][0], rel=1e-6)
    _, spec_m = eng.render(d, engine.PREC_MIXED)
    assert spec_m[0] == pytest.approx(g[f"{name}_spec"][0], rel=FLUX_RTOL_MIXED)


@pytest.mark.parametrize("k,name", [(0, "a05_i120_345"), (1, "a09375_i25_86")])
def test_batch_dumps_match_reference(eng, k, name):
    """The batched configuration's two dumps (a = 0.5 and a = 0.9375), one
    reference image each: FP64 at the parity bar; both mixed forms within
    the flux bar."""
    from raptor_gb300 import engine, workloads
    g = load_golden("batch_dumps_g256.npz")
    d = workloads.batch_dumps(256)[k]
    gid = _grid(eng, d)
    desc = _desc(g[f"{name}_params"], gid)
    img, spec = eng.render(desc, engine.PREC_FP64)
    assert_fp64_parity(img, g[f"{name}_img"], name)
    assert spec[0] == pytest.approx(g[f"{name}_spec"][0], rel=1e-6)
    for prec in (engine.PREC_MIXED, engine.PREC_MIXED_DF):
        _, sm = eng.render(desc, prec)
        assert sm[0] == pytest.approx(g[f"{name}_spec"][0], rel=FLUX_RTOL_MIXED), prec


@pytest.mark.parametrize("name", ["r0_i50_rk4", "r0_i130_rk2"])
def test_nonzero_r0_matches_reference(eng, name):
    """R0 = 0.3 in the dump header (r = R0 + exp(x1)): FP64 at the parity bar,
    both mixed forms within the flux bar."""
    from raptor_gb300 import engine
    from tests.golden.make_golden import r0_dump
    g = load_golden("r0_g64.npz")
    d = r0_dump()
    desc = _desc(g[f"{name}_params"], _grid(eng, d))
    img, spec = eng.render(desc, engine.PREC_FP64)
    assert_fp64_parity(img, g[f"{name}_img"], name)
    assert spec[0] == pytest.approx(g[f"{name}_spec"][0], rel=1e-6)
    for prec in (engine.PREC_MIXED, engine.PREC_MIXED_DF):
        _, sm = eng.render(desc, prec)
        assert sm[0] == pytest.approx(g[f"{name}_spec"][0], rel=FLUX_RTOL_MIXED), prec


def test_fp64_matches_port_and_step_counts(eng, torus64):
    """Step and sample counters agree with the oracle's, ray by ray in sum."""
    from oracle import port
    from raptor_gb300 import engine
    gid = _grid(eng, torus64)
    d = engine.image_desc(20, 20, [230e9, 86e9], grid=gid, inclination=45.0)
    img, _ = eng.render(d, engine.PREC_FP64)
    st = eng.stats()
    sc = port.Scene(torus64.geom, torus64.prims, 20, 20, inclination=45.0)
    ref, _, rs = sc.render([230e9, 86e9], with_stats=True)
    assert_fp64_parity(img.reshape(-1, 2)[:, 0], ref[:, 0], "f0")
    assert_fp64_parity(img.reshape(-1, 2)[:, 1], ref[:, 1], "f1")
    assert abs(st["steps"] - int(rs["steps"].sum())) <= 0.001 * st["steps"]
    assert abs(st["rt_calls"] - int(rs["rt_calls"].sum())) <= 0.001 * st["rt_calls"]


def test_mixed_flux_within_1e4(eng, torus256):
    from raptor_gb300 import engine
    g = load_golden("img100_g256.npz")
    gid = _grid(eng, torus256)
    img, spec = eng.render(_desc(g["params"], gid), engine.PREC_MIXED)
    ref_flux = g["spec"][0]
    assert abs(spec[0] - ref_flux) / ref_flux <= FLUX_RTOL_MIXED
    err = pixel_errors(img, g["img"])
    assert np.median(err) < 1e-4


@pytest.mark.parametrize("integrator", [4, 2])
def test_mixed_df_against_fp64_and_reference(eng, torus256, integrator):
    """Mixed-DF form (double-float geodesic on the FP32 pipes, FP32 transfer):
    total flux within the mixed form's 1e-4 of the reference; the image
    agrees with the FP64 form pixel by pixel as closely as the mixed form
    does (its error is the FP32 transfer's, not the geodesic's), and the
    geodesic itself follows the FP64 one: same step and sample counts to
    0.1 %, the same null-condition drift."""
    from raptor_gb300 import engine
    g = load_golden("img100_g256.npz")
    gid = _grid(eng, torus256)
    params = np.array(g["params"])
    params[4] = integrator
    desc = _desc(params, gid)
    i64, s64 = eng.render(desc, engine.PREC_FP64)
    st64 = eng.stats()
    imx, smx = eng.render(desc, engine.PREC_MIXED)
    idf, sdf = eng.render(desc, engine.PREC_MIXED_DF)
    stdf = eng.stats()
    if integrator == 4:
        assert abs(sdf[0] - g["spec"][0]) / g["spec"][0] <= FLUX_RTOL_MIXED
    assert abs(sdf[0] - s64[0]) / s64[0] <= FLUX_RTOL_MIXED
    err_df = pixel_errors(idf, i64)
    err_mx = pixel_errors(imx, i64)
    assert np.median(err_df) <= 2 * np.median(err_mx) + 1e-7
    assert abs(stdf["steps"] - st64["steps"]) <= 1e-3 * st64["steps"]
    assert abs(stdf["rt_samples"] - st64["rt_samples"]) <= 1e-3 * st64["rt_samples"]
    assert stdf["rays"] == i64.size and stdf["n_nonfinite"] == 0
    assert stdf["kk_max"] <= 1.01 * st64["kk_max"] + 1e-12


def test_deterministic(eng, torus64):
    from raptor_gb300 import engine
    gid = _grid(eng, torus64)
    d = engine.image_desc(24, 24, [230e9], grid=gid)
    a, sa = eng.render(d, engine.PREC_FP64)
    b, sb = eng.render(d, engine.PREC_FP64)
    assert np.array_equal(a, b) and np.array_equal(sa, sb)


def test_batch_equals_single_images(eng, torus64):
    """Images of different sizes, angles and frequencies in one launch give
    what they give alone.  A batch whose widest image has two frequencies runs
    the two-frequency kernel instantiation, whose FMA contraction may differ
    from the one-frequency kernel's, so agreement is at the FP64 parity bar;
    batches of one-frequency images use the same instantiation and agree
    exactly."""
    from raptor_gb300 import engine
    gid = _grid(eng, torus64)
    descs = [engine.image_desc(17, 9, [230e9], grid=gid, inclination=30.0),
             engine.image_desc(8, 12, [86e9, 345e9], grid=gid, inclination=150.0, m_unit=5e18),
             engine.image_desc(5, 5, [230e9], grid=gid, inclination=90.0, integrator=engine.RK2)]
    batch, bspec = eng.render(descs, engine.PREC_FP64)
    off = soff = 0
    for d in descs:
        one, ospec = eng.render(d, engine.PREC_FP64)
        assert_fp64_parity(batch[off:off + one.size], one, "batch image")
        np.testing.assert_allclose(bspec[soff:soff + d.n_freq], ospec, rtol=1e-9)
        off += one.size
        soff += d.n_freq
    same_nf = [descs[0], descs[2]]
    for prec in (engine.PREC_FP64, engine.PREC_MIXED):
        batch, _ = eng.render(same_nf, prec)
        a, _ = eng.render(same_nf[0], prec)
        b, _ = eng.render(same_nf[1], prec)
        assert np.array_equal(batch, np.concatenate([a, b]))


def test_sample_pool_matches_in_place(eng, torus64, torus256):
    """The FP64 form's pooled kernel (samples evaluated 32 at a time from a
    per-warp pool, applied by their rays in step order) and the in-place
    kernel run the same arithmetic per ray: same step and sample counts, and
    the same bits where the compiler emits the same FMA contractions in both
    kernels - the 1-, 2- and 4-frequency instantiations.  The 8-frequency
    instantiations (images with 5-8 frequencies) are separate compilations
    whose last bits may differ; they agree to 1e-12.  Cases: one frequency,
    five, RK2, the log-polar camera, a mixed batch, and a 256x256 image whose
    warps leave the emitting region at different steps."""
    from raptor_gb300 import engine
    ref = engine.Engine(no_sample_pool=1)
    try:
        g64, g256 = _grid(eng, torus64), _grid(eng, torus256)
        r64, r256 = ref.upload_grid(torus64.geom, torus64.prims), ref.upload_grid(torus256.geom, torus256.prims)
        cases = [
            lambda g, h: engine.image_desc(64, 64, [230e9], grid=g, inclination=60.0),
            lambda g, h: engine.image_desc(24, 20, [86e9, 140e9, 230e9, 345e9, 690e9], grid=g, inclination=35.0),
            lambda g, h: engine.image_desc(32, 32, [230e9], grid=g, inclination=120.0, integrator=engine.RK2),
            lambda g, h: engine.image_desc(32, 32, [230e9], grid=g, inclination=17.0, camera=engine.CAM_LOG),
            lambda g, h: [engine.image_desc(17, 9, [230e9], grid=g, inclination=30.0),
                          engine.image_desc(8, 12, [86e9, 345e9], grid=g, inclination=150.0, m_unit=5e18),
                          engine.image_desc(40, 40, [230e9], grid=h, inclination=75.0)],
            lambda g, h: engine.image_desc(256, 256, [230e9], grid=h, inclination=60.0),
        ]
        for k, mk in enumerate(cases):
            a, sa = eng.render(mk(g64, g256), engine.PREC_FP64)
            st_a = eng.stats()
            b, sb = ref.render(mk(r64, r256), engine.PREC_FP64)
            st_b = ref.stats()
            descs = mk(g64, g256)
            if max(d.n_freq for d in (descs if isinstance(descs, list) else [descs])) <= 4:
                assert np.array_equal(a, b, equal_nan=True), f"case {k}: pooled and in-place images differ"
                assert np.array_equal(sa, sb, equal_nan=True), f"case {k}: spectra differ"
            else:
                np.testing.assert_allclose(a, b, rtol=1e-12, atol=0, err_msg=f"case {k}")
                np.testing.assert_allclose(sa, sb, rtol=1e-12, atol=0, err_msg=f"case {k}")
            for key in ("steps", "rt_calls", "rt_samples", "rays", "max_ray_steps"):
                assert st_a[key] == st_b[key], f"case {k}: {key} {st_a[key]} != {st_b[key]}"
    finally:
        ref.close()


def test_range_render_is_a_slice(eng, torus64):
    from raptor_gb300 import engine
    gid = _grid(eng, torus64)
    d = engine.image_desc(16, 16, [230e9], grid=gid)
    full, _ = eng.render(d, engine.PREC_FP64)
    part, _ = eng.render(d, engine.PREC_FP64, ray_begin=37, ray_count=100)
    assert np.array_equal(part[37:137], full[37:137])
    assert not np.any(part[:37]) and not np.any(part[137:])


def test_invalid_arguments_are_rejected(eng, torus64):
    from raptor_gb300 import engine
    gid = _grid(eng, torus64)
    for bad_grid in (-1, 16):  # outside 0..RAPTOR_MAX_GRIDS-1
        with pytest.raises(engine.EngineError):
            eng.render(engine.image_desc(4, 4, [230e9], grid=bad_grid))
    with pytest.raises(engine.EngineError):
        eng.render(engine.image_desc(4, 4, [230e9], grid=gid, camera=7))
    with pytest.raises(engine.EngineError):
        eng.render(engine.image_desc(4, 4, [230e9], grid=gid), 3)  # unknown precision
    with pytest.raises(engine.EngineError):
        eng.render(engine.image_desc(4, 4, [230e9], grid=gid, integrator=3))
    with pytest.raises(engine.EngineError):
        eng.render(engine.image_desc(0, 4, [230e9], grid=gid))
    bad = torus64.prims.copy()
    bad[0, 3, 3] = np.nan
    with pytest.raises(engine.EngineError):
        eng.upload_grid(torus64.geom, bad)
    # the context stays usable after rejected calls
    img, _ = eng.render(engine.image_desc(4, 4, [230e9], grid=gid))
    assert np.all(np.isfinite(img))


@pytest.mark.parametrize("incl", [60.0, 17.0])
def test_1024_on_512_against_reference(eng, incl):
    """Full-size images (the 1024x1024 headline workload): the reference rendered the
    1024x1024 image of the 512x512 torus here with 8 threads; the fixture keeps
    its flux and a strided 17,190-pixel subsample."""
    from raptor_gb300 import engine, synth
    g = load_golden("img1024_g512_sub.npz")
    from tests.golden.make_golden import prim_checksum
    d = synth.make_torus(n1=512, n2=512)
    np.testing.assert_allclose(prim_checksum(d.prims), g["prim_checksum"], rtol=1e-12)
    gid = eng.upload_grid(d.geom, d.prims)
    desc = engine.image_desc(1024, 1024, [230e9], grid=gid, inclination=incl)
    tag = f"i{int(incl)}"
    img, spec = eng.render(desc, engine.PREC_FP64)
    assert_fp64_parity(img[g[f"{tag}_sub_pixels"]], g[f"{tag}_sub_vals"], f"1024 {tag} subsample")
    assert abs(spec[0] - g[f"{tag}_spec"][0]) / g[f"{tag}_spec"][0] <= 1e-6
    mimg, mspec = eng.render(desc, engine.PREC_MIXED)
    assert abs(mspec[0] - g[f"{tag}_spec"][0]) / g[f"{tag}_spec"][0] <= FLUX_RTOL_MIXED
    _, dspec = eng.render(desc, engine.PREC_MIXED_DF)
    assert abs(dspec[0] - g[f"{tag}_spec"][0]) / g[f"{tag}_spec"][0] <= FLUX_RTOL_MIXED


@pytest.mark.parametrize("w,h,nf", [(1, 1, 1), (1, 7, 2), (5, 1, 3), (16, 16, 8)])
def test_edge_shapes_match_port(eng, torus64, w, h, nf):
    """Degenerate and ragged image shapes (single pixel, single row, single
    column) and the largest frequency count, against the oracle port: FP64 at
    the parity bar, the two mixed forms within 1e-4 in flux wherever the
    image is not empty."""
    from oracle import port
    from raptor_gb300 import engine
    freqs = list(np.geomspace(86e9, 690e9, nf))
    desc = engine.image_desc(w, h, freqs, grid=_grid(eng, torus64), inclination=70.0, cam_size_x=12.0,
                             cam_size_y=12.0)
    img, spec = eng.render(desc, engine.PREC_FP64)
    assert img.shape == (w * h * nf,) and spec.shape == (nf,)
    ref, _ = port.Scene(torus64.geom, torus64.prims, w, h, inclination=70.0, cam_size_x=12.0,
                        cam_size_y=12.0).render(freqs)
    assert_fp64_parity(img, ref.ravel(), f"{w}x{h}x{nf}")
    np.testing.assert_allclose(spec, ref.sum(axis=0), rtol=1e-6)
    for prec in (engine.PREC_MIXED, engine.PREC_MIXED_DF):
        _, sm = eng.render(desc, prec)
        for f in range(nf):
            if spec[f] > 0:
                assert abs(sm[f] - spec[f]) <= FLUX_RTOL_MIXED * spec[f], (prec, f)
