"""The algebraic forms the FP64 transfer sample and the FP64 adjoint use
(csrc/transfer.cuh fluid_fast and rt_terms_fp64, csrc/vjp_common.cuh
thetae_log_derivs_fp64, csrc/vjp.cu sample_freq), restated in numpy and
checked against the direct formulas of get_fluid_params
(raptor_harm_model.c:230-276), pitch_angle (radiative_transfer.c:32-47)
and the thermal-synchrotron emissivity (j_nu.c:130-153) over the ranges
HARM data reach.  The GPU parity tests check the kernels' images; this test
pins the rewrites themselves, so a wrong identity fails on the CPU with the
term that broke."""
import numpy as np

RNG = np.random.default_rng(7)
N = 100_000
TINY = 1e-20
MP_ME = 1836.15267247


def _rbeta_direct(uu, bsq, rh, rl):
    beta = uu * (4.0 / 3.0 - 1.0) / (0.5 * (bsq + TINY))
    b2 = beta * beta
    trat = rh * b2 / (1.0 + b2) + rl / (1.0 + b2)
    gam = 0.5 * ((1.0 + 2.0 / 3.0 * (trat + 1.0) / (trat + 2.0)) + 4.0 / 3.0)
    return beta, b2, trat, gam, (gam - 1.0) * MP_ME / (1.0 + trat)


def _rbeta_fast(uu, bsq, rh, rl):
    h = uu * (2.0 / 3.0)
    D = bsq + TINY
    h2, D2 = h * h, D * D
    Q = h2 + D2
    A = rh * h2 + rl * D2 + Q
    C = A + Q
    iAC = 1.0 / (A * C)
    gam = 0.5 * ((1.0 + 2.0 / 3.0 * (A * A * iAC)) + 4.0 / 3.0)
    return gam, (gam - 1.0) * MP_ME * (Q * C * iAC), (h2, D2, Q, A, C)


def _draw():
    uu = 10 ** RNG.uniform(-12, 1, N)
    bsq = 10 ** RNG.uniform(-25, 1, N)
    rho = 10 ** RNG.uniform(-8, 0, N)
    rh = RNG.uniform(1, 100, N)
    rl = RNG.uniform(1, 10, N)
    return uu, bsq, rho, rh, rl


def test_fluid_u0_from_one_rsqrt():
    """u^0 = sqrt(P), 1/u^0 = rsqrt(P), Vfac = w rsqrt(P) with w = 1 + |V.V|
    and P = -g^00 w, against Vfac = sqrt(-1/g^00 w), u^0 = -Vfac g^00."""
    g00 = -(1.0 + RNG.uniform(0, 8, N))  # g^tt = -(1 + 2r/Sigma)
    vv = RNG.uniform(-0.9, 5.0, N)
    vfac = np.sqrt(-1.0 / g00 * (1.0 + np.abs(vv)))
    u0 = -vfac * g00
    w = 1.0 + np.abs(vv)
    p = -g00 * w
    iu0 = 1.0 / np.sqrt(p)
    assert np.max(np.abs(w * iu0 / vfac - 1)) < 1e-15
    assert np.max(np.abs(p * iu0 / u0 - 1)) < 1e-15
    assert np.max(np.abs(iu0 * u0 - 1)) < 1e-15


def test_rbeta_quotients_from_one_reciprocal():
    """(trat + 1)/(trat + 2) = A/C and 1/(1 + trat) = Q/A: Theta_e's unit
    agrees with the direct R-beta formula to rounding, from beta -> 0 to
    beta -> infinity."""
    uu, bsq, _, rh, rl = _draw()
    _, _, _, gam0, tu0 = _rbeta_direct(uu, bsq, rh, rl)
    gam1, tu1, _ = _rbeta_fast(uu, bsq, rh, rl)
    assert np.max(np.abs(gam1 / gam0 - 1)) < 2e-15
    assert np.max(np.abs(tu1 / tu0 - 1)) < 4e-15


def test_thetae_log_derivs_closed_form():
    """thetae_log_derivs_fp64's forms of d ln Theta_e / d(rho, u, R_high,
    R_low) against the direct chain rule and against central differences of
    ln Theta_e itself."""
    uu, bsq, rho, rh, rl = _draw()
    beta, b2, t, gam, _ = _rbeta_direct(uu, bsq, rh, rl)
    i1b2 = 1.0 / (1.0 + b2)
    dlntu = (1.0 / 3.0) / ((t + 2.0) ** 2) / (gam - 1.0) - 1.0 / (1.0 + t)
    dt_dlnb = 2.0 * b2 * (rh - rl) * i1b2 * i1b2
    direct = [-1.0 / rho, (1.0 + dlntu * dt_dlnb) / uu, dlntu * b2 * i1b2, dlntu * i1b2]

    _, _, (h2, D2, Q, A, C) = _rbeta_fast(uu, bsq, rh, rl)
    ce = C * (C + 2.0 * A)
    z = 1.0 / (Q * A * ce)
    iq = z * A * ce
    dlntu_f = -(z * Q * Q) * (A * (3.0 * A + 2.0 * Q) + Q * Q)
    dt_f = 2.0 * (rh - rl) * h2 * D2 * (iq * iq)
    fast = [-1.0 / rho, (1.0 + dlntu_f * dt_f) / uu, dlntu_f * h2 * iq, dlntu_f * D2 * iq]
    for k in range(4):
        scale = np.abs(direct[k]).max()
        assert np.max(np.abs(fast[k] - direct[k])) <= 1e-14 * scale, k

    # against central differences of ln Theta_e = ln(u/rho) + ln(unit(u, R_h, R_l))
    m = slice(0, 2000)

    def ln_th(u, r, a, b):
        return np.log(u / r) + np.log(_rbeta_direct(u, bsq[m], a, b)[4])

    for k, (du, dr, dh, dl) in enumerate(((0, 1, 0, 0), (1, 0, 0, 0), (0, 0, 1, 0), (0, 0, 0, 1))):
        eps = 1e-6
        args_p = [uu[m] * (1 + du * eps), rho[m] * (1 + dr * eps), rh[m] * (1 + dh * eps), rl[m] * (1 + dl * eps)]
        args_m = [uu[m] * (1 - du * eps), rho[m] * (1 - dr * eps), rh[m] * (1 - dh * eps), rl[m] * (1 - dl * eps)]
        base = [uu[m], rho[m], rh[m], rl[m]][[1, 0, 2, 3][k]]
        fd = (ln_th(*args_p) - ln_th(*args_m)) / (2 * eps * base)
        scale = np.abs(fd).max()
        assert np.max(np.abs(fast[k][m] - fd)) <= 1e-6 * scale, k


def test_emission_prefactor_and_root_tangents():
    """j's prefactor n_e sqrt(2) pi nu_s / (3 K2) with K2 = 2 Theta^2 equals
    n_e sqrt(2) pi (2/9) nu_c sin(theta) / 6; the tangents of X^1/3 and
    X^1/6 through 1/X = nu_s / nu_p equal the derivatives of cbrt and sqrt;
    1/nu_p^2 = (1/(k.u))^2 / nu^2 and the pitch cosine from 1/(k.u |B|)."""
    th = 10 ** RNG.uniform(-3, 3, N)
    nuc = 10 ** RNG.uniform(3, 9, N)
    sth = RNG.uniform(1e-6, 1, N)
    ne = 10 ** RNG.uniform(0, 8, N)
    nus = (2.0 / 9.0) * nuc * th * th * sth
    pre0 = ne * (np.sqrt(2.0) * np.pi) * nus / (3.0 * (2.0 * th * th))
    pre1 = ne * (np.sqrt(2.0) * np.pi / 6.0 * (2.0 / 9.0)) * (nuc * sth)
    assert np.max(np.abs(pre1 / pre0 - 1)) < 4e-15

    ku = -(10 ** RNG.uniform(-3, 3, N))
    nu = 10 ** RNG.uniform(9, 12, N)
    nup = -ku * nu
    x = nup * (1.0 / nus)
    ix = nus * (-(1.0 / ku) * (nu * (1.0 / (nu * nu))))
    assert np.max(np.abs(ix * x - 1)) < 8e-16
    cb = np.cbrt(x)
    d_cb = cb * ix / 3.0
    assert np.max(np.abs(d_cb / ((1.0 / 3.0) * x ** (-2.0 / 3.0)) - 1)) < 1e-13
    sv = np.sqrt(cb)
    d_sq = 0.5 * sv * (cb * cb * ix)
    assert np.max(np.abs(d_sq / (0.5 / sv) - 1)) < 1e-13
    inup2 = (1.0 / ku) ** 2 * (1.0 / (nu * nu))
    assert np.max(np.abs(inup2 * nup * nup - 1)) < 2e-15

    bn = 10 ** RNG.uniform(-6, 2, N)
    kdb = RNG.uniform(-1, 1, N) * np.abs(ku) * bn
    ikb = 1.0 / (ku * bn)
    cos0 = kdb / (np.abs(ku) * bn)
    assert np.max(np.abs(kdb * np.abs(ikb) - cos0)) < 4e-16
    assert np.max(np.abs(ikb * bn * ku - 1)) < 4e-16
