"""Synthetic torus generator and the HARM / model.in formats."""
import numpy as np
import pytest

from raptor_gb300 import harm, synth


def test_torus_satisfies_euler_equation():
    ell = synth.torus_ell(0.9375, 12.0)
    for r, th in [(8.0, 1.4), (12.0, 1.57), (15.0, 1.2), (20.0, 1.8)]:
        res = synth.euler_residual(np.float64(r), np.float64(th), 0.9375, ell)
        assert all(abs(x) < 1e-8 for x in res)


def test_pressure_maximum_at_rmax():
    ell = synth.torus_ell(0.5, 12.0)
    rs = np.linspace(9, 15, 601)
    lnh = synth._lnh_unnormalised(rs, np.pi / 2, 0.5, ell)
    assert rs[np.argmax(lnh)] == pytest.approx(12.0, abs=0.02)


def test_plasma_beta_normalisation(torus64):
    ex = torus64.extras
    bsq = np.einsum("...i,...i->...", ex["bcon"], ex["bcov"])
    # before noise: max p_gas / max p_mag = 100; noise moves u by a few percent
    pg = (4 / 3 - 1) * torus64.prims[1]
    ratio = pg.max() / (0.5 * bsq).max()
    assert 80 < ratio < 125


def test_velocity_primitives_reconstruct_unit_four_velocity(torus64):
    """utilde -> u^mu as get_fluid_params does it gives u.u = -1 and matches
    the generator's u^mu."""
    g, gi, _ = synth.mks_metric(torus64.extras["x1"], torus64.extras["x2"], torus64.geom.a, torus64.geom.hslope)
    V = np.moveaxis(torus64.prims[2:5], 0, -1)
    VdotV = np.einsum("...ij,...i,...j->...", g[..., 1:, 1:], V, V)
    vfac = np.sqrt(-1.0 / gi[..., 0, 0] * (1.0 + np.abs(VdotV)))
    u = np.empty(V.shape[:-1] + (4,))
    u[..., 0] = -vfac * gi[..., 0, 0]
    u[..., 1:] = V - vfac[..., None] * gi[..., 0, 1:]
    norm = np.einsum("...ij,...i,...j->...", g, u, u)
    np.testing.assert_allclose(norm, -1.0, atol=1e-10)
    np.testing.assert_allclose(u, torus64.extras["ucon"], rtol=1e-9, atol=1e-12)


def test_noise_stream_is_stable():
    z = synth.normal_stream(12345, 6)
    z2 = synth.normal_stream(12345, 6)
    assert np.array_equal(z, z2)
    big = synth.normal_stream(3, 200000)
    assert abs(big.mean()) < 0.01 and abs(big.std() - 1) < 0.01


def test_dump_round_trip(tmp_path, torus64):
    p = tmp_path / "d.dump"
    harm.write_dump(p, torus64)
    d = harm.read_dump(p)
    assert np.array_equal(d.prims, torus64.prims)
    assert d.geom.n1 == 64 and d.geom.startx1 == torus64.geom.startx1 and d.geom.a == torus64.geom.a


def test_dump_reader_rejects_bad_input(tmp_path, torus64):
    p = tmp_path / "d.dump"
    harm.write_dump(p, torus64)
    lines = open(p).read().splitlines()
    (tmp_path / "trunc.dump").write_text("\n".join(lines[:100]) + "\n")
    with pytest.raises(harm.DumpFormatError):
        harm.read_dump(tmp_path / "trunc.dump")
    with pytest.raises(harm.DumpFormatError):
        harm.read_dump(p, n1=32, n2=32)
    bad = lines[:]
    f = bad[5].split()
    f[4] = "nan"
    bad[5] = " ".join(f)
    (tmp_path / "nan.dump").write_text("\n".join(bad) + "\n")
    with pytest.raises(harm.DumpFormatError):
        harm.read_dump(tmp_path / "nan.dump")


def test_model_in_round_trip(tmp_path):
    m = harm.ModelIn(IMG_WIDTH=123, STEPSIZE=0.025, M_UNIT=3.5e19)
    m.write(tmp_path / "model.in")
    assert harm.ModelIn.read(tmp_path / "model.in") == m
