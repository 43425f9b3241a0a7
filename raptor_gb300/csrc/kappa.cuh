// Kappa-distribution synchrotron emissivity and absorptivity: the fits of
// Pandya et al. (2016) that the reference carries as
// emission_coeff_kappa_FIT and absorption_coeff_kappa_FIT (j_nu.c:28-106),
// with kappa = 3.5 as hard-coded there.  The reference's emission_coeff
// (j_nu.c:20-26) calls the thermal fits; an image selects these instead
// with raptor_image_desc.emission = RAPTOR_EMISSION_KAPPA, as a user of the
// reference would by calling them from emission_coeff.  FP64 form only.
//
// The constants of the fits (gamma functions of kappa, powers of 3 and pi)
// are formed on the host in FP64 (DevImage.kap).  The powers of X = nu/nu_s
// and the fits' smooth-maximum blends (J_low^-x + J_high^-x)^(-1/x) are
// evaluated in the log domain: one log of X per frequency and exps of
// linear combinations, instead of the reference's eight pow() calls - equal
// to rounding.  The absorptivity's Gauss hypergeometric function (GSL's
// gsl_sf_hyperg_2F1 in the reference, j_nu.c:85-96) depends on Theta_e
// only, so it is evaluated once per sample: by Pfaff's transformation and
// the power series for |z| <= 1, and by the reference's connection formula
// with the power series for |z| > 1 (coefficients in kappa_tables.inc,
// generated exactly by gen_kappa_tables.py).
#pragma once
#include <cuda_runtime.h>

#include "fp32_math.cuh"
#include "fp64_math.cuh"
#include "image_desc.cuh"

namespace raptor {

#include "kappa_tables.inc"

// The FP64 functions are templates: T = double in the FP64 sample
// (transfer.cuh, rt_terms_fp64), T = an FP64 dual number in the FP64
// adjoint's sample (vjp.cu), whose values then follow the same operations.

// sum_n C[n] x^n by Horner's rule (80 terms, 0 <= x <= 1/2).
template <class T>
__device__ __forceinline__ T kappa_series(const double* __restrict__ C, const T& x) {
    T s = T(__ldg(&C[79]));
#pragma unroll 8
    for (int n = 78; n >= 0; --n) s = fma(s, x, __ldg(&C[n]));
    return s;
}

// 2F1(kappa - 1/3, kappa + 1; kappa + 2/3; -kappa Theta_e), the reference's
// hyp2F1 (j_nu.c:78-96); 0 where it returns 0 (|z| = 1).
template <class T>
__device__ __forceinline__ T kappa_hyp2f1(const KappaConst& k, const T& thetae) {
    const double a = kKappa - 1.0 / 3.0, b = kKappa + 1.0;
    const T z = -kKappa * thetae;
    if (fabs(z) == 1.0) return T(0.0);
    if (fabs(z) > 1.0) {
        // (1-z)^-a G1 2F1(a, c-b; a-b+1; w) + (1-z)^-b G2 2F1(b, c-a; b-a+1; w),
        // w = 1/(1-z); the first 2F1 is (1-w)^-a, so its term is G1 (-z)^-a
        const T omz = 1.0 - z;
        const T w = recip(omz);
        return k.g1 * pow(-z, -a) + k.g2 * pow(omz, -b) * kappa_series(kKappaConn, w);
    }
    // Pfaff: (1-z)^-a 2F1(a, c-b; c; z/(z-1))
    const T omz = 1.0 - z;
    return pow(omz, -a) * kappa_series(kKappaPfaff, z * recip(z - 1.0));
}

// The per-sample part of the kappa coefficients at frequency-independent
// plasma quantities: B (G), cosine of the pitch angle, Theta_e, n_e.
template <class T>
struct KappaSampleT {
    T fj, fa;             // the fits' prefactors: n_e e^2 nu_c sin / c and n_e e / (B sin)
    T inus;               // 1 / nu_s, nu_s = nu_c sin (Theta_e kappa)^2
    T ln_alow_s;          // ln of A_low's Theta_e-dependent factor, hyp2F1 included
    T ln_ahigh_s;         // ln of A_high's
    bool emits;           // not at a clamped pitch angle (|cos| = 1)
    bool absorbs;         // and hyp2F1 defined (|z| != 1)
};
using KappaSample = KappaSampleT<double>;

template <class T>
__device__ __forceinline__ KappaSampleT<T> kappa_sample(const KappaConst& k, const T& B, const T& cosp,
                                                        const T& thetae, const T& ne) {
    KappaSampleT<T> s;
    const T nuc = B * (kECharge / (2.0 * CUDART_PI * kEMass * kC));
    const T sth = sqrt(1.0 - cosp * cosp);
    s.fj = (ne * (kECharge * kECharge) * nuc * sth) * (1.0 / kC);
    const T wk = thetae * kKappa;
    s.inus = recip(nuc * sth * (wk * wk));
    s.fa = ne * kECharge * recip(B * sth);
    s.emits = fabs(cosp) != 1.0;
    const T h = kappa_hyp2f1(k, thetae);
    s.absorbs = h != 0.0;
    const T lnwk = log(wk);
    s.ln_alow_s = k.ln_alow - (16.0 / 3.0 - kKappa) * lnwk + log(h);
    s.ln_ahigh_s = k.ln_ahigh - 5.0 * lnwk;
    return s;
}

// (e^(-x u) + e^(-x v))^(-1/x) for u, v the logs of the two fits.
template <class T>
__device__ __forceinline__ T kappa_blend(const T& u, const T& v, double x) {
    return exp(-log(fast_exp(-x * u) + fast_exp(-x * v)) / x);
}

// j_nu and a_nu at plasma-frame frequency nup (j_nu.c:28-106).
template <class T>
__device__ __forceinline__ void kappa_coeffs(const KappaConst& k, const KappaSampleT<T>& s, const T& nup, T& j,
                                             T& a) {
    j = T(0.0);
    a = T(0.0);
    if (nup == 1.0 || !s.emits) return;
    const T lnX = log(nup * s.inus);
    j = s.fj * kappa_blend(k.ln_jlow + lnX * (1.0 / 3.0), k.ln_jhigh - (kKappa - 2.0) / 2.0 * lnX, k.xj);
    if (s.absorbs)
        a = s.fa * kappa_blend(s.ln_alow_s - (5.0 / 3.0) * lnX, s.ln_ahigh_s - (3.0 + kKappa) / 2.0 * lnX, k.xa);
}

// ----------------------------------------------------------------- FP32
// The same fits for the FP32 transfer samples of the mixed and mixed-DF
// forms, from the FP32 copies of the constants (DevImage.kapf).  The
// emissivity is carried without its e2_c = e^2/c factor, as the FP32
// thermal emissivity is (transfer.cuh), and the blends
// (e^(-x u) + e^(-x v))^(-1/x) are formed around the larger exponent, so
// that e^(-x u) cannot overflow FP32's range (it would near x u = -88).

// Templates as the FP64 functions are: T = float in the FP32 samples
// (transfer.cuh), T = an FP32 dual number in the mixed forms' adjoints
// (vjp_df.cu).

// sum_n C[n] x^n by Horner's rule (40 terms, 0 <= x <= 1/2).
template <class T>
__device__ __forceinline__ T kappa_series_f(const float* __restrict__ C, const T& x) {
    T s = T(__ldg(&C[39]));
#pragma unroll 8
    for (int n = 38; n >= 0; --n) s = fma(s, x, __ldg(&C[n]));
    return s;
}

// kappa_hyp2f1 in FP32
template <class T>
__device__ __forceinline__ T kappa_hyp2f1_f(const KappaConstF& k, const T& thetae) {
    const float a = (float)(kKappa - 1.0 / 3.0), b = (float)(kKappa + 1.0);
    const T z = -(float)kKappa * thetae;
    if (fabs(z) == 1.0f) return T(0.0f);
    const T omz = 1.0f - z;
    if (fabs(z) > 1.0f)
        return k.g1 * pow(-z, -a) + k.g2 * pow(omz, -b) * kappa_series_f(kKappaConnF, fdiv(T(1.0f), omz));
    return pow(omz, -a) * kappa_series_f(kKappaPfaffF, fdiv(z, z - 1.0f));
}

template <class T>
struct KappaSampleFT {
    T fj;            // n_e nu_c sin: the emissivity's prefactor over e2_c
    T fa;            // n_e e / (B sin)
    T inus;          // 1 / nu_s
    T ln_alow_s, ln_ahigh_s;
    bool emits, absorbs;
};
using KappaSampleF = KappaSampleFT<float>;

template <class T>
__device__ __forceinline__ KappaSampleFT<T> kappa_sample_f(const KappaConstF& k, const T& B, const T& cosp,
                                                           const T& thetae, const T& ne) {
    KappaSampleFT<T> s;
    const T nuc = B * (float)(kECharge / (2.0 * CUDART_PI * kEMass * kC));
    const T sth = fsqrt(1.0f - cosp * cosp);
    s.fj = ne * nuc * sth;
    const T wk = thetae * (float)kKappa;
    s.inus = fdiv(T(1.0f), nuc * sth * (wk * wk));
    s.fa = ne * (float)kECharge * fdiv(T(1.0f), B * sth);
    s.emits = fabs(cosp) != 1.0f;
    const T h = kappa_hyp2f1_f(k, thetae);
    s.absorbs = h != 0.0f;
    const T lnwk = log(wk);
    s.ln_alow_s = k.ln_alow - (float)(16.0 / 3.0 - kKappa) * lnwk + log(h);
    s.ln_ahigh_s = k.ln_ahigh - 5.0f * lnwk;
    return s;
}

// (e^(-x u) + e^(-x v))^(-1/x) = e^(-(m + ln(1 + e^-|x (u - v)|)) / x), m = max(-x u, -x v)
template <class T>
__device__ __forceinline__ T kappa_blend_f(const T& u, const T& v, float x) {
    const T m = fmax(-x * u, -x * v);
    return exp(-fdiv(m + log1p(exp(-fabs(x * (u - v)))), T(x)));
}

// j_nu / e2_c and a_nu at plasma-frame frequency nup
template <class T>
__device__ __forceinline__ void kappa_coeffs_f(const KappaConstF& k, const KappaSampleFT<T>& s, const T& nup, T& j,
                                               T& a) {
    j = T(0.0f);
    a = T(0.0f);
    if (nup == 1.0f || !s.emits) return;
    const T lnX = log(nup * s.inus);
    j = s.fj * kappa_blend_f(k.ln_jlow + lnX * (1.0f / 3.0f), k.ln_jhigh - (float)((kKappa - 2.0) / 2.0) * lnX, k.xj);
    if (s.absorbs)
        a = s.fa * kappa_blend_f(s.ln_alow_s - (5.0f / 3.0f) * lnX,
                                 s.ln_ahigh_s - (float)((3.0 + kKappa) / 2.0) * lnX, k.xa);
}

}  // namespace raptor
