"""Seeded synthetic HARM-format GRMHD dumps (the reference's sample dump is
not distributed, so every workload here is synthetic).

The dump is a 2D axisymmetric Fishbone-Moncrief torus on the modified
Kerr-Schild (MKS) grid that the reference samples:

* grid: x1 = ln r uniform on [ln Rin, ln Rout] (R0 = 0), x2 uniform on
  [0, 1], theta = pi x2 + (1 - hslope)/2 sin(2 pi x2) (metric.c:98 of the
  reference), cell-centred values at x = startx + (i + 1/2) dx, as Xtoij
  (grmhd.c:46-71) assumes;
* torus: constant u^t u_phi angular momentum, pressure maximum at r_max,
  inner edge r_in, polytrope p = K rho^gamma with gamma = 4/3, rho_max = 1;
* velocity primitives: HARM's relative 4-velocity
  utilde^i = u^i - u^t g^{ti}/g^{tt}, which get_fluid_params inverts
  (raptor_harm_model.c:235-242);
* field: poloidal, from A_phi = max(rho/rho_max - 0.2, 0),
  B^1 = -d_2 A / sqrt(-g), B^2 = d_1 A / sqrt(-g), scaled so that
  max(p_gas) / max(b^2/2) = beta (100);
* a seeded log-normal perturbation exp(sigma z) of rho and u (sigma = 0.04).

The torus equations are derived here from the relativistic Euler equation
for circular flow (d_i ln h = 1/2 d_i g_{mu nu} u^mu u^nu); the derivation is
checked numerically by tests/test_synth.py.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

# primitive order of the HARM dump and of the reference's p[] array
# (raptor_harm_model.h:63-70)
PRIM_NAMES = ("rho", "u", "u1", "u2", "u3", "B1", "B2", "B3")
NPRIM = 8


@dataclasses.dataclass
class TorusSpec:
    n1: int = 256
    n2: int = 256
    a: float = 0.9375
    hslope: float = 0.3
    r_in: float = 6.0
    r_max: float = 12.0
    gamma: float = 4.0 / 3.0
    beta: float = 100.0
    rout: float = 40.0
    rin_factor: float = 0.98  # Rin = rin_factor * r_horizon
    noise: float = 0.04
    seed: int = 12345


@dataclasses.dataclass
class GridGeom:
    """Grid geometry, as read from the dump header (raptor_harm_model.c:90-135)."""
    n1: int
    n2: int
    startx1: float
    startx2: float
    dx1: float
    dx2: float
    a: float
    hslope: float
    R0: float = 0.0
    Rin: float = 0.0
    Rout: float = 0.0
    gam: float = 4.0 / 3.0

    @property
    def stopx1(self) -> float:
        return self.startx1 + self.n1 * self.dx1

    @property
    def stopx2(self) -> float:
        return self.startx2 + self.n2 * self.dx2


@dataclasses.dataclass
class Dump:
    geom: GridGeom
    prims: np.ndarray  # float64 [8][n1][n2], primitive-major (HARM order)
    extras: dict       # ucon, ucov, bcon, bcov, gdet, x1, x2, r, th (for the ASCII dump)


def horizon_radius(a: float) -> float:
    return 1.0 + math.sqrt(1.0 - a * a)


def _bl_quantities(r, th, a):
    s = np.sin(th)
    c = np.cos(th)
    sig = r * r + a * a * c * c
    dlt = r * r - 2.0 * r + a * a
    A = (r * r + a * a) ** 2 - dlt * a * a * s * s
    return s, c, sig, dlt, A


def _circular_state(r, th, a, ell):
    """ZAMO decomposition of the constant-ell circular flow.

    With e^{2 nu} = Sigma Delta / A, e^{2 psi} = A sin^2 / Sigma,
    omega = 2 a r / A and X = (gamma v)^2, the definition ell = u^t u_phi
    gives X^2 + X = ell^2 e^{2(nu - psi)}."""
    s, c, sig, dlt, A = _bl_quantities(r, th, a)
    e2nu = sig * dlt / A
    e2psi = A * s * s / sig
    om = 2.0 * a * r / A
    X = 0.5 * (-1.0 + np.sqrt(1.0 + 4.0 * ell * ell * e2nu / e2psi))
    lorentz = np.sqrt(1.0 + X)
    ut = lorentz / np.sqrt(e2nu)
    uph = ut * om + np.sqrt(X) / np.sqrt(e2psi)
    return X, lorentz, ut, uph, e2nu, om


def _lnh_unnormalised(r, th, a, ell):
    """ln h up to a constant: ln u^t - X - omega ell."""
    X, lorentz, ut, uph, e2nu, om = _circular_state(r, th, a, ell)
    return np.log(ut) - X - om * ell


def _bl_metric_dd(r, th, a):
    s, c, sig, dlt, A = _bl_quantities(r, th, a)
    g = np.zeros(np.broadcast(r, th).shape + (4, 4))
    g[..., 0, 0] = -(1.0 - 2.0 * r / sig)
    g[..., 0, 3] = g[..., 3, 0] = -2.0 * a * r * s * s / sig
    g[..., 1, 1] = sig / dlt
    g[..., 2, 2] = sig
    g[..., 3, 3] = A * s * s / sig
    return g


def euler_residual(r, th, a, ell, h=1e-5):
    """d_i ln h - 1/2 d_i g_{mu nu} u^mu u^nu for i = r, theta (finite
    differences); zero when the torus equations are consistent."""
    X, lorentz, ut, uph, e2nu, om = _circular_state(r, th, a, ell)
    u = np.stack([ut, np.zeros_like(ut), np.zeros_like(ut), uph], axis=-1)
    out = []
    for dr, dth in ((h, 0.0), (0.0, h)):
        dl = (_lnh_unnormalised(r + dr, th + dth, a, ell)
              - _lnh_unnormalised(r - dr, th - dth, a, ell)) / (2 * h)
        dg = (_bl_metric_dd(r + dr, th + dth, a) - _bl_metric_dd(r - dr, th - dth, a)) / (2 * h)
        rhs = 0.5 * np.einsum("...ij,...i,...j->...", dg, u, u)
        out.append(dl - rhs)
    return out


def torus_ell(a: float, r_max: float) -> float:
    """Angular momentum ell = u^t u_phi that puts the pressure maximum of the
    equatorial profile at r_max (d_r ln h = 0 there), by bisection."""
    def dlnh(ell):
        h = 1e-6 * r_max
        return (_lnh_unnormalised(r_max + h, math.pi / 2, a, ell)
                - _lnh_unnormalised(r_max - h, math.pi / 2, a, ell)) / (2 * h)
    lo, hi = 1.0, 20.0
    flo, fhi = dlnh(lo), dlnh(hi)
    if flo * fhi > 0:
        raise ValueError("no pressure maximum bracket for the torus angular momentum")
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        fm = dlnh(mid)
        if (fm > 0) == (flo > 0):
            lo, flo = mid, fm
        else:
            hi = mid
    return 0.5 * (lo + hi)


def mks_theta(x2, hslope):
    return np.pi * x2 + 0.5 * (1.0 - hslope) * np.sin(2.0 * np.pi * x2)


def mks_metric(x1, x2, a, hslope):
    """MKS covariant and contravariant metric (R0 = 0), the same formulas as
    the reference's metric_dd/metric_uu MKS branches (metric.c:94-137,
    207-231), vectorised."""
    r = np.exp(x1)
    th = mks_theta(x2, hslope)
    s = np.sin(th)
    c = np.cos(th)
    rho2 = r * r + a * a * c * c
    hfac = np.pi + (1.0 - hslope) * np.pi * np.cos(2.0 * np.pi * x2)
    shape = np.broadcast(x1, x2).shape
    g = np.zeros(shape + (4, 4))
    g[..., 0, 0] = -1.0 + 2.0 * r / rho2
    g[..., 0, 1] = g[..., 1, 0] = 2.0 * r / rho2 * r
    g[..., 0, 3] = g[..., 3, 0] = -2.0 * a * r * s * s / rho2
    g[..., 1, 1] = (1.0 + 2.0 * r / rho2) * r * r
    g[..., 1, 3] = g[..., 3, 1] = -a * s * s * (1.0 + 2.0 * r / rho2) * r
    g[..., 2, 2] = rho2 * hfac * hfac
    g[..., 3, 3] = s * s * (rho2 + a * a * s * s * (1.0 + 2.0 * r / rho2))
    irho2 = 1.0 / rho2
    gi = np.zeros(shape + (4, 4))
    gi[..., 0, 0] = -1.0 - 2.0 * r * irho2
    gi[..., 0, 1] = gi[..., 1, 0] = 2.0 * irho2
    gi[..., 1, 1] = irho2 * (r * (r - 2.0) + a * a) / (r * r)
    gi[..., 1, 3] = gi[..., 3, 1] = a * irho2 / r
    gi[..., 2, 2] = irho2 / (hfac * hfac)
    gi[..., 3, 3] = irho2 / (s * s)
    gdet = rho2 * s * r * hfac
    return g, gi, gdet


def _splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser (Steele, Lea & Flood 2014), vectorised, wrapping uint64."""
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def normal_stream(seed: int, n: int) -> np.ndarray:
    """n standard normal deviates from a counter-based stream (splitmix64 of
    seed*2^32 + index, Box-Muller), identical on every numpy version and
    platform up to libm rounding."""
    idx = np.arange(2 * ((n + 1) // 2), dtype=np.uint64) + np.uint64(seed) * np.uint64(1 << 32)
    bits = _splitmix64(idx)
    u = ((bits >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
    u1, u2 = u[0::2], u[1::2]
    rad = np.sqrt(-2.0 * np.log(u1))
    z = np.empty(u.size)
    z[0::2] = rad * np.cos(2.0 * np.pi * u2)
    z[1::2] = rad * np.sin(2.0 * np.pi * u2)
    return z[:n]


def make_torus(spec: TorusSpec | None = None, **kw) -> Dump:
    """Build the seeded torus dump described in the module docstring."""
    spec = dataclasses.replace(spec or TorusSpec(), **kw)
    a, hs = spec.a, spec.hslope
    n1, n2 = spec.n1, spec.n2
    Rin = spec.rin_factor * horizon_radius(a)
    startx1 = math.log(Rin)
    dx1 = (math.log(spec.rout) - startx1) / n1
    startx2 = 0.0
    dx2 = 1.0 / n2
    x1 = startx1 + (np.arange(n1) + 0.5) * dx1
    x2 = startx2 + (np.arange(n2) + 0.5) * dx2
    X1, X2 = np.meshgrid(x1, x2, indexing="ij")
    r = np.exp(X1)
    th = mks_theta(X2, hs)

    ell = torus_ell(a, spec.r_max)
    lnh0 = _lnh_unnormalised(spec.r_in, math.pi / 2, a, ell)
    with np.errstate(invalid="ignore"):  # inside the horizon Delta < 0; masked below
        lnh = _lnh_unnormalised(r, th, a, ell) - lnh0
        _, _, ut_c, uph_c, _, _ = _circular_state(r, th, a, ell)
    lnh = np.where(np.isfinite(lnh), lnh, -1.0)
    lnh_max = float(_lnh_unnormalised(spec.r_max, math.pi / 2, a, ell) - lnh0)
    gam = spec.gamma
    inside = (r >= spec.r_in) & (lnh > 0.0)
    hh = np.exp(np.where(inside, lnh, 0.0))
    hmax = math.exp(lnh_max)
    kappa = (hmax - 1.0) * (gam - 1.0) / gam
    rho_t = np.where(inside, ((hh - 1.0) * (gam - 1.0) / (kappa * gam)) ** (1.0 / (gam - 1.0)), 0.0)
    u_t = np.where(inside, kappa * rho_t ** gam / (gam - 1.0), 0.0)

    rho_floor = 1e-6 * r ** -1.5
    u_floor = 1e-8 * r ** -2.5
    rho = np.maximum(rho_t, rho_floor)
    uu = np.maximum(u_t, u_floor)

    g, gi, gdet = mks_metric(X1, X2, a, hs)
    # torus four-velocity: (u^t, 0, 0, u^phi) in BL == KS == MKS components here
    # normal observer elsewhere: u^mu = n^mu = (1/alpha, -alpha g^{ti}) with alpha = 1/sqrt(-g^tt)
    alpha = 1.0 / np.sqrt(-gi[..., 0, 0])
    ucon = np.zeros(r.shape + (4,))
    ucon[..., 0] = np.where(inside, ut_c, 1.0 / alpha)
    ucon[..., 1] = np.where(inside, 0.0, -alpha * gi[..., 0, 1])
    ucon[..., 2] = 0.0
    ucon[..., 3] = np.where(inside, uph_c, -alpha * gi[..., 0, 3])
    # relative 4-velocity primitives utilde^i = u^i - u^t g^{ti}/g^{tt}
    util = ucon[..., 1:] - ucon[..., :1] * gi[..., 0, 1:] / gi[..., 0, 0:1]
    util = np.where(inside[..., None], util, 0.0)

    # poloidal field from A_phi = max(rho/rho_max - 0.2, 0)
    Aphi = np.maximum(rho_t / 1.0 - 0.2, 0.0)
    dA1 = np.gradient(Aphi, dx1, axis=0)
    dA2 = np.gradient(Aphi, dx2, axis=1)
    Bp = np.zeros(r.shape + (3,))
    Bp[..., 0] = -dA2 / gdet
    Bp[..., 1] = dA1 / gdet
    ucov = np.einsum("...ij,...j->...i", g, ucon)
    bt = np.einsum("...i,...i->...", Bp, ucov[..., 1:])
    bcon = np.zeros_like(ucon)
    bcon[..., 0] = bt
    bcon[..., 1:] = (Bp + bt[..., None] * ucon[..., 1:]) / ucon[..., :1]
    bcov = np.einsum("...ij,...j->...i", g, bcon)
    bsq = np.einsum("...i,...i->...", bcon, bcov)
    pmax = float(np.max((gam - 1.0) * u_t))
    bmax = float(np.max(0.5 * bsq))
    norm = math.sqrt(pmax / (spec.beta * bmax)) if bmax > 0 else 0.0
    Bp *= norm
    bcon *= norm
    bcov *= norm

    z = normal_stream(spec.seed, 2 * r.size).reshape((2,) + r.shape)
    rho = rho * np.exp(spec.noise * z[0])
    uu = uu * np.exp(spec.noise * z[1])

    prims = np.empty((NPRIM, n1, n2), dtype=np.float64)
    prims[0] = rho
    prims[1] = uu
    prims[2:5] = np.moveaxis(util, -1, 0)
    prims[5:8] = np.moveaxis(Bp, -1, 0)
    geom = GridGeom(n1=n1, n2=n2, startx1=startx1, startx2=startx2, dx1=dx1, dx2=dx2,
                    a=a, hslope=hs, R0=0.0, Rin=Rin, Rout=spec.rout, gam=gam)
    extras = dict(x1=X1, x2=X2, r=r, th=th, ucon=ucon, ucov=ucov, bcon=bcon, bcov=bcov,
                  gdet=gdet, ell=ell)
    return Dump(geom=geom, prims=np.ascontiguousarray(prims), extras=extras)
