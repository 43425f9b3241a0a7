// Accuracy of the engine's table-driven fast_exp / fast_sincospi against
// CUDA's exp / sincospi on the GPU (built and run by tests/test_gpu_math.py).
// Prints the maximum ulp difference for each, over arguments covering the
// ranges the geodesic uses (x1 = ln r in [0, 10]; 2 x2 and theta/pi in
// [-0.1, 2.1]) and wider ones.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <vector>

#include "df64.cuh"
#include "fp64_math.cuh"

__global__ void eval(const double* x, int n, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s0, c0, s1, c1;
    raptor::fast_sincospi(x[i], &s0, &c0);
    sincospi(x[i], &s1, &c1);
    out[6 * i + 0] = raptor::fast_exp(x[i]);
    out[6 * i + 1] = exp(x[i]);
    out[6 * i + 2] = s0;
    out[6 * i + 3] = s1;
    out[6 * i + 4] = c0;
    out[6 * i + 5] = c1;
}

// The double-float (hi + lo FP32 pairs) exp and sincospi of df64.cuh, and
// DF division, against CUDA's FP64 functions; relative errors.
__global__ void eval_df(const double* x, int n, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xe = fabs(x[i]) * (10.0 / 30.0);  // x1 = ln r in [0, 10]
    const raptor::DF de = raptor::df_const(xe);
    const raptor::DF ds = raptor::df_const(x[i] * (1.0 / 14.0));  // [-2.1, 2.1]
    raptor::DF s0, c0;
    raptor::fast_sincospi(ds, &s0, &c0);
    double s1, c1;
    sincospi(raptor::df_to_double(ds), &s1, &c1);
    const double e1 = exp(raptor::df_to_double(de));
    const raptor::DF q = de / ds;
    out[4 * i + 0] = fabs(raptor::df_to_double(raptor::fast_exp(de)) - e1) / e1;
    out[4 * i + 1] = fabs(raptor::df_to_double(s0) - s1);
    out[4 * i + 2] = fabs(raptor::df_to_double(c0) - c1);
    const double qd = raptor::df_to_double(de) / raptor::df_to_double(ds);
    out[4 * i + 3] = fabs(raptor::df_to_double(q) - qd) / fabs(qd);
}

// fast_rcp (fp64_math.cuh) against the IEEE quotient 1/x
__global__ void eval_rcp(const double* x, int n, double* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[2 * i] = raptor::fast_rcp(x[i]);
    out[2 * i + 1] = 1.0 / x[i];
}

// fdiv / fsqrt (fp32_math.cuh) against IEEE FP32 division and sqrtf
__global__ void eval_f32(const float* a, const float* b, int n, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[4 * i + 0] = raptor::fdiv(a[i], b[i]);
    out[4 * i + 1] = a[i] / b[i];
    out[4 * i + 2] = raptor::fsqrt(fabsf(a[i]));
    out[4 * i + 3] = sqrtf(fabsf(a[i]));
}

// f32_of (fp32_math.cuh) against the IEEE double -> float conversion
__global__ void eval_f2f(const double* x, int n, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[2 * i] = raptor::f32_of(x[i]);
    out[2 * i + 1] = (float)x[i];
}

static double ulpsf(float a, float b) {
    if (a == b) return 0;
    if (!std::isfinite(a) || !std::isfinite(b)) return 1e30;
    int ia, ib;
    memcpy(&ia, &a, 4);
    memcpy(&ib, &b, 4);
    if ((ia < 0) != (ib < 0)) return 1e30;
    return fabs((double)ia - (double)ib);
}

static double ulps(double a, double b) {
    if (a == b) return 0;
    if (!std::isfinite(a) || !std::isfinite(b)) return 1e30;
    long long ia, ib;
    memcpy(&ia, &a, 8);
    memcpy(&ib, &b, 8);
    if ((ia < 0) != (ib < 0)) return fabs(a - b) < 1e-300 ? 0 : 1e30;
    return fabs((double)(ia - ib));
}

int main() {
    const int n = 1 << 21;
    std::vector<double> x(n);
    unsigned long long s = 88172645463325252ull;
    for (int i = 0; i < n; ++i) {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        double u = (s >> 11) * (1.0 / 9007199254740992.0);
        x[i] = (i % 2) ? (-0.1 + 2.2 * u) : (-30.0 + 60.0 * u);
    }
    double *dx, *dout;
    cudaMalloc(&dx, n * sizeof(double));
    cudaMalloc(&dout, 6 * (size_t)n * sizeof(double));
    cudaMemcpy(dx, x.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    eval<<<(n + 255) / 256, 256>>>(dx, n, dout);
    std::vector<double> o(6 * (size_t)n);
    cudaMemcpy(o.data(), dout, o.size() * sizeof(double), cudaMemcpyDeviceToHost);
    double me = 0, ms = 0, mc = 0, abs_s = 0, abs_c = 0;
    for (int i = 0; i < n; ++i) {
        me = fmax(me, ulps(o[6 * i], o[6 * i + 1]));
        ms = fmax(ms, ulps(o[6 * i + 2], o[6 * i + 3]));
        mc = fmax(mc, ulps(o[6 * i + 4], o[6 * i + 5]));
        abs_s = fmax(abs_s, fabs(o[6 * i + 2] - o[6 * i + 3]));
        abs_c = fmax(abs_c, fabs(o[6 * i + 4] - o[6 * i + 5]));
    }
    eval_df<<<(n + 255) / 256, 256>>>(dx, n, dout);
    cudaMemcpy(o.data(), dout, 4 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
    double df_e = 0, df_s = 0, df_c = 0, df_q = 0;
    for (int i = 0; i < n; ++i) {
        df_e = fmax(df_e, o[4 * i]);
        df_s = fmax(df_s, o[4 * i + 1]);
        df_c = fmax(df_c, o[4 * i + 2]);
        if (std::isfinite(o[4 * i + 3])) df_q = fmax(df_q, o[4 * i + 3]);
    }
    // reciprocals over magnitudes 2^-500 .. 2^500 of both signs
    std::vector<double> rx(n);
    for (int i = 0; i < n; ++i) {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        const double u = (s >> 11) * (1.0 / 9007199254740992.0);
        rx[i] = ((s >> 3) & 1 ? -1.0 : 1.0) * ldexp(1.0 + u, (int)((s >> 40) % 1001) - 500);
    }
    const double special[] = {0.0, -0.0, INFINITY, -INFINITY, NAN};
    for (int k = 0; k < 5; ++k) rx[k] = special[k];
    cudaMemcpy(dx, rx.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    eval_rcp<<<(n + 255) / 256, 256>>>(dx, n, dout);
    cudaMemcpy(o.data(), dout, 2 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
    double rcp_u = 0;
    for (int k = 0; k < 4; ++k)  // IEEE's infinities and zeros, signs included
        if (!(o[2 * k] == o[2 * k + 1]) || std::signbit(o[2 * k]) != std::signbit(o[2 * k + 1])) rcp_u = 1e30;
    if (!(o[8] != o[8])) rcp_u = 1e30;  // NaN stays NaN
    for (int i = 5; i < n; ++i) rcp_u = fmax(rcp_u, ulps(o[2 * i], o[2 * i + 1]));
    // FP32 quotients and square roots over magnitudes 2^-149 .. 2^127 of both
    // signs (subnormals included), then IEEE's special cases
    std::vector<float> fa(n), fb(n);
    for (int i = 0; i < n; ++i) {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        const float u = (float)((s >> 40) * (1.0 / 16777216.0));
        fa[i] = ((s >> 3) & 1 ? -1.0f : 1.0f) * ldexpf(1.0f + u, (int)((s >> 8) % 277) - 149);
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        const float v = (float)((s >> 40) * (1.0 / 16777216.0));
        fb[i] = ((s >> 3) & 1 ? -1.0f : 1.0f) * ldexpf(1.0f + v, (int)((s >> 8) % 277) - 149);
    }
    const float sa[] = {0.0f, 1.0f, 0.0f, INFINITY, 3.0f, -0.0f, NAN};
    const float sb[] = {0.0f, 0.0f, 2.0f, 2.0f, INFINITY, 1.0f, 1.0f};
    for (int k = 0; k < 7; ++k) { fa[k] = sa[k]; fb[k] = sb[k]; }
    float *dfa, *dfb, *dfo;
    cudaMalloc(&dfa, n * sizeof(float));
    cudaMalloc(&dfb, n * sizeof(float));
    cudaMalloc(&dfo, 4 * (size_t)n * sizeof(float));
    cudaMemcpy(dfa, fa.data(), n * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(dfb, fb.data(), n * sizeof(float), cudaMemcpyHostToDevice);
    eval_f32<<<(n + 255) / 256, 256>>>(dfa, dfb, n, dfo);
    std::vector<float> fo(4 * (size_t)n);
    cudaMemcpy(fo.data(), dfo, fo.size() * sizeof(float), cudaMemcpyDeviceToHost);
    double div_u = 0, div_u_sub = 0, sqrt_u = 0;
    int special_bad = 0;
    for (int k = 0; k < 7; ++k) {
        const float q = fo[4 * k], qi = fo[4 * k + 1], r = fo[4 * k + 2], ri = fo[4 * k + 3];
        const bool qs = (q == qi && std::signbit(q) == std::signbit(qi)) || (q != q && qi != qi);
        const bool rs = (r == ri && std::signbit(r) == std::signbit(ri)) || (r != r && ri != ri);
        special_bad += !qs + !rs;
    }
    for (int i = 7; i < n; ++i) {
        const float qi = fo[4 * i + 1];
        const double u = ulpsf(fo[4 * i], qi);
        if (fabsf(qi) >= 1.17549435e-38f && fabsf(qi) < 3.0e38f) div_u = fmax(div_u, u);
        else if (fabsf(qi) < 1.17549435e-38f) div_u_sub = fmax(div_u_sub, u);
        sqrt_u = fmax(sqrt_u, ulpsf(fo[4 * i + 2], fo[4 * i + 3]));
    }
    // double -> float over magnitudes 2^-140 .. 2^140 of both signs, exact
    // ties of the FP32 rounding, then zeros, infinities and NaN
    for (int i = 0; i < n; ++i) {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        const double u = (s >> 11) * (1.0 / 9007199254740992.0);
        rx[i] = ((s >> 3) & 1 ? -1.0 : 1.0) * ldexp(1.0 + u, (int)((s >> 40) % 281) - 140);
        if (i % 64 == 1) {  // a tie: 24 significant bits and a half
            long long b;
            memcpy(&b, &rx[i], 8);
            b = (b & ~0x1fffffffll) | 0x10000000ll;
            memcpy(&rx[i], &b, 8);
        }
    }
    const double dspecial[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 3.4028235677973366e38, 1e-40, -1e-39};
    for (int k = 0; k < 8; ++k) rx[k] = dspecial[k];
    cudaMemcpy(dx, rx.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    eval_f2f<<<(n + 255) / 256, 256>>>(dx, n, dfo);
    cudaMemcpy(fo.data(), dfo, 2 * (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
    double f2f_u = 0;
    int f2f_bad = 0, f2f_ties = 0;
    for (int i = 0; i < n; ++i) {
        const float c = fo[2 * i], ci = fo[2 * i + 1];
        const double ax = fabs(rx[i]);
        if (rx[i] != rx[i]) {
            f2f_bad += !std::isinf(c);  // NaN -> infinity
        } else if (ax < 1.1754943508222875e-38) {
            f2f_bad += !(c == 0.0f && std::signbit(c) == std::signbit(rx[i]));  // signed zero
        } else if (std::isinf(ci)) {
            f2f_bad += !(c == ci);
        } else {
            long long b;
            memcpy(&b, &rx[i], 8);
            const bool tie = (b & 0x1fffffffll) == 0x10000000ll;
            const double u = ulpsf(c, ci);
            f2f_ties += tie && u > 0;
            if (!tie) f2f_bad += u > 0;  // equal but at ties
            f2f_u = fmax(f2f_u, u);
        }
    }
    printf("exp_ulp %g sin_ulp %g cos_ulp %g sin_abs %g cos_abs %g df_exp_rel %g df_sin_abs %g df_cos_abs %g "
           "df_div_rel %g rcp_ulp %g fdiv_ulp %g fdiv_sub_ulp %g fsqrt_ulp %g f32_special_bad %d "
           "f2f_ulp %g f2f_bad %d f2f_tie_diffs %d err %s\n",
           me, ms, mc, abs_s, abs_c, df_e, df_s, df_c, df_q, rcp_u, div_u, div_u_sub, sqrt_u, special_bad,
           f2f_u, f2f_bad, f2f_ties, cudaGetErrorString(cudaGetLastError()));
    return 0;
}
