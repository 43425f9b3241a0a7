// Accuracy of the engine's table-driven fast_exp / fast_sincospi against
// CUDA's exp / sincospi on the GPU (built and run by tests/test_gpu_math.py).
// Prints the maximum ulp difference for each, over arguments covering the
// ranges the geodesic uses (x1 = ln r in [0, 10]; 2 x2 and theta/pi in
// [-0.1, 2.1]) and wider ones.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <vector>

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
    printf("exp_ulp %g sin_ulp %g cos_ulp %g sin_abs %g cos_abs %g err %s\n", me, ms, mc, abs_s, abs_c,
           cudaGetErrorString(cudaGetLastError()));
    return 0;
}
