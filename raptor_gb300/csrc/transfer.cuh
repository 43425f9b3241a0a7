// One radiative-transfer sample at the post-step position of a ray:
// get_fluid_params (raptor_harm_model.c:190-320) with Xtoij / bilinear
// interpolation (grmhd.c:35-71), pitch_angle and freq_in_plasma_frame
// (radiative_transfer.c:17-47), thermal synchrotron j_nu and Kirchhoff
// a_nu (j_nu.c:130-153, 188-200) and the tau / I update of
// radiative_transfer.c:71-98.
//
// Two forms share the sampling structure:
//  * rt_sample_fp64 - FP64 throughout, the reference's formulas (pow of
//    1/2, 1/6, 1/3 written as sqrt / cbrt) with fewer divisions: constant
//    divisors folded, a nu formed without B_nu, its edge cases (B_nu
//    underflow) those of the reference's a = j e2_ch / B_nu / e2_c.
//  * rt_sample_fp32 - metric in FP64, then fluid, tetrad projection,
//    emissivity and the tau / I accumulation in FP32 with Neumaier
//    compensated sums.  Emissivity is carried without the e2_c factor and
//    the absorptivity as j_hat (e^x - 1) / nu^2 so every intermediate stays
//    inside FP32's range; e2_c is applied once per ray in FP64.
#pragma once
#include "fp32_math.cuh"
#include "image_desc.cuh"
#include "kappa.cuh"

namespace raptor {

struct CellCoef {
    int base;    // (i * n2 + j): first of the four cells
    double d1, d2;
};

// Xtoij (grmhd.c:46-71): cell-centred index, truncation toward zero,
// clamped to [0, N-2] with del = 0 / 1 at the clamps.  del is formed as
// t - i with t = (x - startx)/dx - 1/2, the reference's
// (x - ((i + 1/2) dx + startx))/dx regrouped.
__device__ __forceinline__ CellCoef cell_coef(const DevImage& im, double x1, double x2) {
    CellCoef cc;
    const double t1 = (x1 - im.startx1) * im.idx1 - 0.5;
    const double t2 = (x2 - im.startx2) * im.idx2 - 0.5;
    int i = (int)t1, j = (int)t2;
    double d1, d2;
    if (i < 0) { i = 0; d1 = 0.0; }
    else if (i > im.n1 - 2) { i = im.n1 - 2; d1 = 1.0; }
    else d1 = t1 - (double)i;
    if (j < 0) { j = 0; d2 = 0.0; }
    else if (j > im.n2 - 2) { j = im.n2 - 2; d2 = 1.0; }
    else d2 = t2 - (double)j;
    if (!chk(i >= 0 && i <= im.n1 - 2 && j >= 0 && j <= im.n2 - 2, im.check_word, kChkCell,
             (long long)i * im.n2 + j))
        i = j = 0;
    cc.base = i * im.n2 + j;
    cc.d1 = d1;
    cc.d2 = d2;
    return cc;
}

__device__ __forceinline__ void load_cell(const double* __restrict__ c, double v[8]) {
    const double2* p = reinterpret_cast<const double2*>(c);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const double2 t = __ldg(p + q);
        v[2 * q] = t.x;
        v[2 * q + 1] = t.y;
    }
}
__device__ __forceinline__ void load_cell(const float* __restrict__ c, float v[8]) {
    const float4* p = reinterpret_cast<const float4*>(c);
    const float4 t0 = __ldg(p), t1 = __ldg(p + 1);
    v[0] = t0.x; v[1] = t0.y; v[2] = t0.z; v[3] = t0.w;
    v[4] = t1.x; v[5] = t1.y; v[6] = t1.z; v[7] = t1.w;
}

// Bilinear interpolation of all eight primitives, coefficient order of
// raptor_harm_model.c:213-216 and term order of grmhd.c:38-41.
template <class T>
__device__ __forceinline__ void interp_prims_at(const T* __restrict__ cells, int n2, int base, T d1, T d2,
                                                T v[8]) {
    const T c0 = (T(1) - d1) * (T(1) - d2), c1 = (T(1) - d1) * d2;
    const T c2 = d1 * (T(1) - d2), c3 = d1 * d2;
    T a[8], b[8], e[8], f[8];
    const T* p = cells + (size_t)base * 8;
    load_cell(p, a);
    load_cell(p + 8, b);
    load_cell(p + (size_t)n2 * 8, e);
    load_cell(p + (size_t)n2 * 8 + 8, f);
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = a[q] * c0 + b[q] * c1 + e[q] * c2 + f[q] * c3;
}
template <class T>
__device__ __forceinline__ void interp_prims(const T* __restrict__ cells, int n2, const CellCoef& cc,
                                             T v[8]) {
    interp_prims_at(cells, n2, cc.base, narrow<T>(cc.d1), narrow<T>(cc.d2), v);
}

template <class T>
struct MetricT {
    T d00, d01, d03, d11, d13, d22, d33;
    T u00, u01, u11, u13, u22, u33;
};

template <class T>
__device__ __forceinline__ MetricT<T> metric_cast(const MetricDD& d, const MetricUU& u) {
    MetricT<T> m;
    m.d00 = (T)d.g00; m.d01 = (T)d.g01; m.d03 = (T)d.g03; m.d11 = (T)d.g11;
    m.d13 = (T)d.g13; m.d22 = (T)d.g22; m.d33 = (T)d.g33;
    m.u00 = (T)u.g00; m.u01 = (T)u.g01; m.u11 = (T)u.g11; m.u13 = (T)u.g13;
    m.u22 = (T)u.g22; m.u33 = (T)u.g33;
    return m;
}

template <class T>
__device__ __forceinline__ void lowerT(const MetricT<T>& g, const T v[4], T out[4]) {
    out[0] = g.d00 * v[0] + g.d01 * v[1] + g.d03 * v[3];
    out[1] = g.d01 * v[0] + g.d11 * v[1] + g.d13 * v[3];
    out[2] = g.d22 * v[2];
    out[3] = g.d03 * v[0] + g.d13 * v[1] + g.d33 * v[3];
}

template <class T>
struct Fluid {
    T ne, thetae, B, bsq;
    T ucon[4], bcon[4];
    T irho;  // 1 / rho
};

// get_fluid_params (raptor_harm_model.c:190-290) from interpolated
// primitives.  Returns false in the sigma = b^2/rho > 1 cut (line 285).
template <class T>
__device__ __forceinline__ bool fluid_from_prims(const T v[8], const MetricT<T>& g, T Ne_unit, T B_unit,
                                                 T r_high, T r_low, Fluid<T>& fl) {
    const T tiny = (T)1.e-20;
    const T rho = v[0], uu = v[1];
    const T V1 = v[2], V2 = v[3], V3 = v[4];
    const T Bp1 = v[5], Bp2 = v[6], Bp3 = v[7];
    fl.ne = rho * Ne_unit;
    // g_ij V^i V^j, i,j = 1..3, with g_12 = g_23 = 0
    const T VdotV = (g.d11 * V1 + T(2) * g.d13 * V3) * V1 + g.d22 * V2 * V2 + g.d33 * V3 * V3;
    const T Vfac = fsqrt(fdiv(T(-1), g.u00) * (T(1) + fabs(VdotV)));
    T* U = fl.ucon;
    U[0] = -Vfac * g.u00;
    U[1] = V1 - Vfac * g.u01;
    U[2] = V2;  // g^{02} = 0
    U[3] = V3;  // g^{03} = 0
    T Ucov[4];
    lowerT(g, U, Ucov);
    const T UdotBp = Ucov[1] * Bp1 + Ucov[2] * Bp2 + Ucov[3] * Bp3;
    T* Bc = fl.bcon;
    const T iU0 = fdiv(T(1), U[0]);
    Bc[0] = UdotBp;
    Bc[1] = (Bp1 + U[1] * UdotBp) * iU0;
    Bc[2] = (Bp2 + U[2] * UdotBp) * iU0;
    Bc[3] = (Bp3 + U[3] * UdotBp) * iU0;
    T Bcov[4];
    lowerT(g, Bc, Bcov);
    const T Bsq = Bc[0] * Bcov[0] + Bc[1] * Bcov[1] + Bc[2] * Bcov[2] + Bc[3] * Bcov[3];
    fl.bsq = Bsq;
    fl.B = fsqrt(Bsq) * B_unit + tiny;
    // R-beta electron temperature, raptor_harm_model.c:262-276
    const T beta = fdiv(uu * (T(4) / T(3) - T(1)), T(0.5) * (Bsq + tiny));
    const T b2 = beta * beta;
    const T i1b2 = fdiv(T(1), T(1) + b2);
    const T trat = r_high * b2 * i1b2 + r_low * i1b2;
    // (trat + 1)/(trat + 2) and 1/(1 + trat) from one division
    const T tp1 = trat + T(1), tp2 = trat + T(2);
    const T itt = fdiv(T(1), tp1 * tp2);
    const T two_temp_gam = T(0.5) * ((T(1) + T(2) / T(3) * (tp1 * tp1 * itt)) + T(4) / T(3));
    const T Thetae_unit = (two_temp_gam - T(1)) * (T)(kPMass / kEMass) * (tp2 * itt);
    const T irho = fdiv(T(1), rho);
    fl.irho = irho;
    T th = (uu * irho) * Thetae_unit;
    if (th < T(0)) th = tiny;
    fl.thetae = th;
    return !(Bsq * irho > T(1));  // the sigma cut, b^2 / rho > 1
}

// get_fluid_params for the FP64 sample and the FP64 adjoint's dual sample
// (T = double or an FP64 dual): fluid_from_prims's quantities from one
// reciprocal square root and two divisions where the template takes a
// square root and six divisions (the FP32 samples of the mixed forms and the
// mixed-DF adjoint keep the template: in FP32 the D^2 of a weak field
// underflows).  With
// w = 1 + |V.V| and P = -g^00 w: u^0 = sqrt(P), the 1/u^0 of b^i is rsqrt(P)
// and Vfac = sqrt(w / -g^00) = w rsqrt(P).  In the R-beta model beta = h / D
// with h = 2u/3 and D = b^2 + tiny, so trat = N / Q with
// N = r_high h^2 + r_low D^2 and Q = h^2 + D^2; with A = N + Q and C = A + Q
// the two quotients the model needs, (trat + 1)/(trat + 2) = A / C and
// 1/(1 + trat) = Q / A, come from one reciprocal of A C.  D^2 >= 1e-40, so
// no product underflows.
template <class T>
__device__ __forceinline__ bool fluid_fast(const T v[8], const MetricT<T>& g, const T& Ne_unit, const T& B_unit,
                                           const T& r_high, const T& r_low, Fluid<T>& fl) {
    const double tiny = 1.e-20;
    const T rho = v[0], uu = v[1];
    const T V1 = v[2], V2 = v[3], V3 = v[4];
    const T Bp1 = v[5], Bp2 = v[6], Bp3 = v[7];
    fl.ne = rho * Ne_unit;
    const T VdotV = (g.d11 * V1 + 2.0 * g.d13 * V3) * V1 + g.d22 * V2 * V2 + g.d33 * V3 * V3;
    const T w = 1.0 + fabs(VdotV);
    const T P = -g.u00 * w;
    const T iU0 = rsqrt(P);
    const T Vfac = w * iU0;
    T* U = fl.ucon;
    U[0] = P * iU0;
    U[1] = V1 - Vfac * g.u01;
    U[2] = V2;  // g^{02} = 0
    U[3] = V3;  // g^{03} = 0
    T Ucov[4];
    lowerT(g, U, Ucov);
    const T UdotBp = Ucov[1] * Bp1 + Ucov[2] * Bp2 + Ucov[3] * Bp3;
    T* Bc = fl.bcon;
    Bc[0] = UdotBp;
    Bc[1] = (Bp1 + U[1] * UdotBp) * iU0;
    Bc[2] = (Bp2 + U[2] * UdotBp) * iU0;
    Bc[3] = (Bp3 + U[3] * UdotBp) * iU0;
    T Bcov[4];
    lowerT(g, Bc, Bcov);
    const T Bsq = Bc[0] * Bcov[0] + Bc[1] * Bcov[1] + Bc[2] * Bcov[2] + Bc[3] * Bcov[3];
    fl.bsq = Bsq;
    fl.B = sqrt(Bsq) * B_unit + tiny;
    // R-beta electron temperature, raptor_harm_model.c:262-276
    const T h = uu * (2.0 / 3.0), D = Bsq + tiny;
    const T h2 = h * h, D2 = D * D;
    const T Q = h2 + D2;
    const T A = r_high * h2 + r_low * D2 + Q;
    const T C = A + Q;
    const T iAC = recip(A * C);
    const T two_temp_gam = 0.5 * ((1.0 + 2.0 / 3.0 * (A * A * iAC)) + 4.0 / 3.0);
    const T Thetae_unit = (two_temp_gam - 1.0) * (kPMass / kEMass) * (Q * C * iAC);
    const T irho = recip(rho);
    fl.irho = irho;
    T th = (uu * irho) * Thetae_unit;
    if (th < 0.0) th = T(tiny);
    fl.thetae = th;
    return !(Bsq * irho > 1.0);  // the sigma cut, b^2 / rho > 1
}

// ---------------------------------------------------------------- FP64 form
// The sample splits into the part that depends only on the post-step point -
// fluid, emissivity and absorptivity, per frequency the optical-depth
// increment nu_p a_nu dl_f and j_nu / nu_p^2 - and the tau / I update that
// depends on the ray's history.  rt_terms_fp64 and rt_apply_fp64 are that
// split; run back to back (rt_sample_fp64) they are the sample of
// radiative_transfer.c:71-98, operation for operation.

// Returns false in the sigma cut (no change to the ray).  Frequencies that do
// not emit get dtau = jn = 0, except where B_nu underflows to 0 (exp overflow
// at very low Theta_e): there the reference gets a = 0 / 0 and tau NaN for the
// rest of the ray, carried here as dtau = NaN.
template <int NF>
__device__ __forceinline__ bool rt_terms_fp64(const DevImage& im, const double y[8], const MksPoint& p,
                                              double adl, double (&dtau)[NF], double (&jn)[NF]) {
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        dtau[f] = 0.0;
        jn[f] = 0.0;
    }
    MetricDD gd;
    MetricUU gu;
    mks_metric(p, im.geo, gd, gu);
    const MetricT<double> g = metric_cast<double>(gd, gu);
    const CellCoef cc = cell_coef(im, y[1], y[2]);
    double v[8];
    interp_prims(im.cells64, im.n2, cc, v);
    Fluid<double> fl;
    if (!fluid_fast<double>(v, g, im.Ne_unit, im.B_unit, im.r_high, im.r_low, fl)) return false;

    const double k[4] = {y[4], y[5], y[6], y[7]};
    double kd[4];
    lowerT(g, k, kd);
    const double* U = fl.ucon;
    const double* Bc = fl.bcon;
    const double kU = kd[0] * U[0] + kd[1] * U[1] + kd[2] * U[2] + kd[3] * U[3];
    // pitch_angle (radiative_transfer.c:32-47): cosine, clamped to [-1, 1].
    // 1/(k.u |B|) gives the cosine's 1/(|k.u| |B|) (|B| > 0) and 1/(k.u).
    const double Bn = fl.B * im.inv_B_unit;
    const double ikB = recip(kU * Bn);
    double pitch = (kd[0] * Bc[0] + kd[1] * Bc[1] + kd[2] * Bc[2] + kd[3] * Bc[3]) * fabs(ikB);
    if (fabs(pitch) > 1.0) pitch /= fabs(pitch);
    if (im.emission == kEmissionKappa) {
        // the kappa fits (kappa.cuh) in place of the thermal ones:
        // dtau = nu_p a_nu dl_f and j_nu / nu_p^2, radiative_transfer.c:87-90
        const KappaSample ks = kappa_sample(im.kap, fl.B, pitch, fl.thetae, fl.ne);
        const double ikU = ikB * Bn;
        const double ikU2 = ikU * ikU;
#pragma unroll 1
        for (int f = 0; f < NF; ++f) {
            if (f >= im.nfreq) break;
            double nup = -kU * im.freq[f];
            if (nup <= 0.0) nup = 1.0;
            double j, a;
            kappa_coeffs(im.kap, ks, nup, j, a);
            dtau[f] = nup * a * (adl * im.rg_over_nu[f]);
            jn[f] = j * (ikU2 * im.inv_freq2[f]);  // 1/nu_p^2 where j != 0 (nu_p not the sentinel)
        }
        return true;
    }
    const double sth = sqrt(1.0 - pitch * pitch);
    const double nuc = fl.B * (kECharge / (2.0 * CUDART_PI * kEMass * kC));
    const double nus = (2.0 / 9.0) * nuc * fl.thetae * fl.thetae * sth;
    const bool emits = (fabs(sth) >= 1.e-10) && (fl.thetae > 1e-4);
    // j = n_e sqrt(2) pi nu_s / (3 K2) F(X) e2_c with K2 = 2 Theta^2: the
    // frequency-independent factor n_e sqrt(2) pi (2/9) nu_c sin(theta) e2_c / 6
    // once per sample (nu_s / Theta^2 taken as (2/9) nu_c sin(theta))
    const double jpre = fl.ne * (1.4142135623730951 * CUDART_PI / 6.0 * (2.0 / 9.0) * kE2C) * (nuc * sth);
    // h nu / (k T) = nu h / (m_e c^2 Theta_e)
    const double hkt = (kPlanck / (kEMass * kC * kC)) * recip(fl.thetae);
    // 1/nu_s, and 1/nu_p^2 = (1/(k.u))^2 / nu^2, once per sample
    const double inus = recip(nus);
    const double ikU = ikB * Bn;
    const double ikU2 = ikU * ikU;
    // one copy of the frequency body (5 frequencies: 7 % faster than unrolled)
#pragma unroll 1
    for (int f = 0; f < NF; ++f) {
        if (f >= im.nfreq) break;
        // freq_in_plasma_frame with nu scaling folded: -(u . k_d) nu
        double nup = -kU * im.freq[f];
        if (nup <= 0.0) nup = 1.0;
        // B_nu = 2 nu^3 / c^2 / (e^{h nu / k T} - 1); ex = e^{h nu / k T} - 1
        const double ex = fast_exp(hkt * nup) - 1.0;
        if (emits && nup != 1.0) {
            const double dlf = adl * im.rg_over_nu[f];
            const double X = nup * inus;
            const double cb = cbrt(X);
            // X^1/2 + 2^(11/12) X^1/6 = X^1/6 (X^1/3 + 2^(11/12)): one square root
            const double sq = sqrt(cb) * (cb + 1.8877486253633869);
            const double j = jpre * (sq * sq) * fast_exp(-cb);
            const double inup2 = ikU2 * im.inv_freq2[f];
            // a nu = j e2_ch / B_nu / e2_c nu = j (e2_ch c^2 / (2 e2_c)) ex / nu^2: inf where
            // B_nu underflows (ex = inf), NaN where j = 0 there too, as j e2_ch / B_nu
            dtau[f] = j * (kE2CH * kC * kC / (2.0 * kE2C)) * ex * inup2 * dlf;
            jn[f] = j * inup2;
        } else if (!(ex < CUDART_INF)) {
            // j = 0 and B_nu underflowed to 0: the reference's a = 0 / 0
            dtau[f] = __longlong_as_double(0x7ff8000000000000ll);
        }
    }
    return true;
}

// The ordered part: tau += dtau, then I += j/nu_p^2 e^-tau dl_f inside the
// tau gate (radiative_transfer.c:89-95).  The two sums are rounded on their
// own (as the reference, C without FMA contraction, does), so no kernel can
// fuse them with the products that formed their terms.
template <int NF>
__device__ __forceinline__ void rt_apply_fp64(const DevImage& im, double adl, const double (&dtau)[NF],
                                              const double (&jn)[NF], double (&tau)[NF], double (&I)[NF]) {
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        if (f >= im.nfreq) break;
        if (dtau[f] == 0.0 && jn[f] == 0.0) continue;  // no emission: tau and I unchanged
        tau[f] = __dadd_rn(tau[f], dtau[f]);
        const double dI = jn[f] * fast_exp(-tau[f]) * (adl * im.rg_over_nu[f]);
        if (tau[f] < 6.907755278982137 && !(tau[f] < 0.0)) I[f] = __dadd_rn(I[f], dI);  // log(1000)
    }
}

template <int NF>
__device__ __forceinline__ bool rt_sample_fp64(const DevImage& im, const double y[8], const MksPoint& p,
                                               double adl, double (&tau)[NF], double (&I)[NF]) {
    double dtau[NF], jn[NF];
    if (!rt_terms_fp64<NF>(im, y, p, adl, dtau, jn)) return false;
    rt_apply_fp64<NF>(im, adl, dtau, jn, tau, I);
    return true;
}

// ------------------------------------------------------------- FP32 form
__device__ __forceinline__ void neumaier_add(float& s, float& c, float x) {
    const float t = s + x;
    if (fabsf(s) >= fabsf(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

// The FP32 sample in three parts: the frequency-independent terms
// (sample_common_fp32: fluid, k.u, pitch angle, emissivity prefactors), one
// frequency's order-free terms (sample_freq_fp32: d tau and j / nu_p^2) and
// their ordered application to tau and I (sample_apply_fp32).  The in-place
// samples run them in one loop (rt_sample_fp32_core); the mixed-DF form's
// sample pool evaluates the first two for 32 rays at once and applies the
// third in each ray's step order - the same operations either way.
struct SampleF32 {
    float kU, nus, jpre, xpre;
    bool emits;
    bool kappa;       // the kappa fits (kappa.cuh) in place of the thermal ones
    KappaSampleF ks;  // their per-sample part
};

// false at the sigma cut (no sample)
__device__ __forceinline__ bool sample_common_fp32(const DevImage& im, const MetricT<float>& g, const float v[8],
                                                   const float k[4], SampleF32& sc) {
    Fluid<float> fl;
    if (!fluid_from_prims(v, g, im.ne_unit_f, im.b_unit_f, im.r_high_f, im.r_low_f, fl)) return false;
    float kd[4];
    lowerT(g, k, kd);
    const float* U = fl.ucon;
    const float* Bc = fl.bcon;
    sc.kU = kd[0] * U[0] + kd[1] * U[1] + kd[2] * U[2] + kd[3] * U[3];
    float pitch = fdiv(kd[0] * Bc[0] + kd[1] * Bc[1] + kd[2] * Bc[2] + kd[3] * Bc[3],
                       fabsf(sc.kU) * (fl.B * im.inv_b_unit_f));
    if (fabsf(pitch) > 1.0f) pitch = copysignf(1.0f, pitch);  // pitch / |pitch|
    sc.kappa = im.emission == kEmissionKappa;
    if (sc.kappa) {
        sc.ks = kappa_sample_f(im.kapf, fl.B, pitch, fl.thetae, fl.ne);
        return true;
    }
    const float sth = fsqrt(1.0f - pitch * pitch);
    const float nuc = (float)(kECharge / (2.0 * CUDART_PI * kEMass * kC)) * fl.B;
    sc.nus = (2.0f / 9.0f) * nuc * fl.thetae * fl.thetae * sth;
    sc.emits = (fabsf(sth) >= 1.e-10f) && (fl.thetae > 1e-4f);
    // j / e2_c = n_e sqrt(2) pi nu_s / (3 K2) F(X) with K2 = 2 Theta^2, nu_s = (2/9) nu_c Theta^2 sin
    sc.jpre = fl.ne * (float)(1.4142135623730951 * CUDART_PI / 27.0) * nuc * sth;
    sc.xpre = fdiv((float)(kPlanck / (kEMass * kC * kC)), fl.thetae);  // h nu / (k T) per Hz
    return true;
}

// Frequency f: d tau and q = j / nu_p^2 (in units of e2_c), false where it
// does not emit (tau and I stay as they are).  dlf = |d lambda| R_g / nu_f.
__device__ __forceinline__ bool sample_freq_fp32(const DevImage& im, const SampleF32& sc, int f, float dlf,
                                                 float& dtau, float& q) {
    float nup = -sc.kU * im.freq_f[f];
    if (nup <= 0.0f) nup = 1.0f;
    if (sc.kappa) {
        // dtau = nu_p a_nu dl_f and j_nu / nu_p^2, radiative_transfer.c:87-90
        float j, a;
        kappa_coeffs_f(im.kapf, sc.ks, nup, j, a);
        if (j == 0.0f && a == 0.0f) return false;  // as the FP64 sample: tau and I unchanged
        q = fdiv(fdiv(j, nup), nup);
        dtau = nup * a * dlf;
        return true;
    }
    if (!(sc.emits && nup != 1.0f)) return false;
    const float X = fdiv(nup, sc.nus);
    const float cb = cbrtf(X);
    const float sq = fsqrt(cb) * (cb + 1.8877486f);  // X^1/2 + 2^(11/12) X^1/6
    const float jh = sc.jpre * (sq * sq) * expf(-cb);
    q = fdiv(fdiv(jh, nup), nup);
    dtau = q * expm1f(sc.xpre * nup) * (float)(kE2CH * kC * kC * 0.5) * dlf;
    return true;
}

// tau += d tau, then I += q e^-tau dlf unless tau is past the ln 1000 gate
// (radiative_transfer.c:87-98), both compensated
__device__ __forceinline__ void sample_apply_fp32(float dtau, float q, float dlf, float& tau, float& tauc, float& I,
                                                  float& Ic) {
    neumaier_add(tau, tauc, dtau);
    const float t = tau + tauc;
    const float dI = q * expf(-t) * dlf;
    if (t < 6.9077553f && !(t < 0.0f)) neumaier_add(I, Ic, dI);
}

// The in-place FP32 sample from the metric, the interpolated primitives and
// the photon wave vector in FP32.  dlf_of(f) gives |d lambda| R_g / nu_f.
template <int NF, class DlfOf>
__device__ __forceinline__ bool rt_sample_fp32_core(const DevImage& im, const MetricT<float>& g, const float v[8],
                                                    const float k[4], DlfOf dlf_of, float (&tau)[NF],
                                                    float (&tauc)[NF], float (&I)[NF], float (&Ic)[NF]) {
    SampleF32 sc;
    if (!sample_common_fp32(im, g, v, k, sc)) return false;
    // one copy of the frequency body (mixed-DF, 5 frequencies: 12 % faster)
#pragma unroll 1
    for (int f = 0; f < NF; ++f) {
        if (f >= im.nfreq) break;
        const float dlf = dlf_of(f);
        float dtau, q;
        if (sample_freq_fp32(im, sc, f, dlf, dtau, q)) sample_apply_fp32(dtau, q, dlf, tau[f], tauc[f], I[f], Ic[f]);
    }
    return true;
}

// The FP32 samples' metric (metric.c:94-137, 207-231 as mks_metric) in FP32
// from the point's quantities rounded to FP32 (r, sin theta, 1/Sigma,
// theta', Sigma, 1/r', 1/theta', 1/sin theta) and the spin and R0: it feeds
// only the FP32 fluid and tetrad projection.
struct PointF32 {
    float r, s, iS, thp, Sg, irp, ithp, isn;
};

__device__ __forceinline__ MetricT<float> metric_f32(const PointF32& q, float a, float a2, float R0) {
    const float r = q.r, s = q.s, irho2 = q.iS;
    const float s2 = s * s;
    const float rfac = r - R0;
    const float hfac = q.thp;
    const float rho2 = q.Sg;
    const float z = 2.0f * r * irho2;
    const float ir = (R0 == 0.0f) ? q.irp : fdiv(1.0f, r);
    MetricT<float> g;
    g.d00 = -1.0f + z;
    g.d01 = z * rfac;
    g.d03 = -a * z * s2;
    g.d11 = (1.0f + z) * rfac * rfac;
    g.d13 = -a * s2 * (1.0f + z) * rfac;
    g.d22 = rho2 * hfac * hfac;
    g.d33 = s2 * (rho2 + a2 * s2 * (1.0f + z));
    g.u00 = -1.0f - z;
    g.u01 = 2.0f * irho2;
    g.u11 = irho2 * (r * (r - 2.0f) + a2) * (ir * ir);
    g.u13 = a * irho2 * ir;
    g.u22 = irho2 * (q.ithp * q.ithp);
    g.u33 = irho2 * (q.isn * q.isn);
    return g;
}

// Mixed form: the cell coefficients from the FP64 geodesic state, the
// metric in FP32 from the FP64 point rounded (computing it in FP64 and
// rounding it took some 30 FP64-pipe instructions per sample, run with the
// warp's non-sampling lanes idle; the roundings are f32_of's, on the
// integer pipes, for the same reason).
template <int NF>
__device__ __forceinline__ bool rt_sample_fp32(const DevImage& im, const double y[8], const MksPoint& p,
                                               double adl, float (&tau)[NF], float (&tauc)[NF],
                                               float (&I)[NF], float (&Ic)[NF]) {
    const PointF32 q{f32_of(p.r),  f32_of(p.s),   f32_of(p.iS),   f32_of(p.thp),
                     f32_of(p.Sg), f32_of(p.irp), f32_of(p.ithp), f32_of(p.isn)};
    const MetricT<float> g = metric_f32(q, im.geo_df.a.hi, im.geo_df.a2.hi, im.geo_df.R0.hi);
    const CellCoef cc = cell_coef(im, y[1], y[2]);
    float v[8];
    interp_prims(im.cells32, im.n2, cc, v);
    const float k[4] = {f32_of(y[4]), f32_of(y[5]), f32_of(y[6]), f32_of(y[7])};
    return rt_sample_fp32_core<NF>(im, g, v, k, [&](int f) { return f32_of(adl * im.rg_over_nu[f]); }, tau,
                                   tauc, I, Ic);
}

}  // namespace raptor
