"""The one-pass adjoint's record-and-close scheme (csrc/vjp_df.cu
vjp_f32_body, csrc/vjp.cu consume_term), restated in numpy.

Per ray and frequency the reference's transfer recurrence
(radiative_transfer.c:88-95) is I = sum_k g_k S_k exp(-tau_k) with
tau_k = sum_{m<=k} delta_m and g_k the ln 1000 gate, so that
dI/dS_k = g_k exp(-tau_k) and dI/ddelta_k = -(I - I_<k).  A sample's
gradient term along a direction x is therefore
G_k = sum_f w_f (g exp(-tau) dS/dx - (I_f - I_<k,f) ddelta/dx).

The two-pass adjoint evaluates it with I from a forward render.  The one
pass writes, for each sample inside some frequency's gate, the gated part
and per frequency (I_<k, w ddelta/dx), and closes the record with the ray's
own I when the ray ends.  Checked here: the closed records reproduce the
two-pass terms; a sample past every frequency's gate has a term of exactly
zero when I is the ray's own running sum (tau never decreases, so nothing
after it adds to I; with I from a separate forward render, whose sums round
differently, the term is rounding noise instead), which is why it writes no
record; and the two sensitivities agree with central differences of I at
fixed gates.
"""
import numpy as np

LN1000 = 6.907755278982137


def _ray(rng, k, nf):
    """Emission S >= 0 and optical depths delta >= 0 along one ray, some
    rays thick enough to close the gates part-way."""
    s = rng.lognormal(0.0, 1.0, (k, nf))
    d = rng.lognormal(np.log(rng.uniform(0.01, 0.5)), 1.0, (k, nf))
    return s, d


def _transfer(s, d):
    """tau, gate, the prefix I_<k and the total I, as the kernels accumulate
    them (tau += delta first, then the gated contribution; I is the running
    sum's last value, the ray's own I the one pass closes its records with)."""
    tau = np.cumsum(d, axis=0)
    g = tau < LN1000
    contrib = np.where(g, s * np.exp(-tau), 0.0)
    run = np.cumsum(contrib, axis=0)
    before = np.vstack([np.zeros((1, s.shape[1])), run[:-1]])
    return tau, g, before, run[-1]


def test_closed_records_equal_two_pass_terms():
    rng = np.random.default_rng(11)
    n_rec = n_samples = 0
    for _ in range(200):
        k, nf = int(rng.integers(5, 400)), int(rng.integers(1, 6))
        s, d = _ray(rng, k, nf)
        tau, g, before, total = _transfer(s, d)
        w = rng.normal(size=nf)
        ds, dd = rng.normal(size=(k, nf)), rng.normal(size=(k, nf))
        e = np.exp(-tau)
        # two passes: I from the forward render (here the same sums)
        two = (w * (np.where(g, e, 0.0) * ds - (total - before) * dd)).sum(axis=1)
        # one pass: records for samples inside some gate, closed at the end
        live = g.any(axis=1)
        gated = (w * np.where(g, e, 0.0) * ds).sum(axis=1)
        coeff = w * dd
        one = np.where(live, gated - (coeff * (total - before)).sum(axis=1), 0.0)
        scale = np.abs(two).max()
        assert np.abs(one - two).max() <= 1e-12 * scale
        # past every gate the two-pass term is exactly zero: nothing is lost
        assert np.all(two[~live] == 0.0)
        n_rec += int(live.sum())
        n_samples += k
    assert 0 < n_rec < n_samples  # some rays closed their gates


def test_sensitivities_match_central_differences():
    rng = np.random.default_rng(5)
    s, d = _ray(rng, 60, 2)
    d *= 0.2
    tau, g, before, total = _transfer(s, d)

    def intensity(s_, d_):
        t = np.cumsum(d_, axis=0)
        return np.where(g, s_ * np.exp(-t), 0.0).sum(axis=0)  # gates held fixed

    for k in (0, 17, 59):
        for f in range(2):
            h = 1e-6 * s[k, f]
            sp, sm = s.copy(), s.copy()
            sp[k, f] += h
            sm[k, f] -= h
            fd = (intensity(sp, d)[f] - intensity(sm, d)[f]) / (2 * h)
            assert np.isclose(fd, g[k, f] * np.exp(-tau[k, f]), rtol=1e-7)
            h = 1e-6 * d[k, f]
            dp, dm = d.copy(), d.copy()
            dp[k, f] += h
            dm[k, f] -= h
            fd = (intensity(s, dp)[f] - intensity(s, dm)[f]) / (2 * h)
            assert np.isclose(fd, -(total[f] - before[k, f]), rtol=1e-6)
