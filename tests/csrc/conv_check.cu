// Checks the integer-pipe FP64 <-> FP32 conversions of mac_internal.cuh against the hardware
// conversions, bit for bit: random doubles across the whole exponent range, rounding ties, the
// FP32 range limits, signed zeros, subnormals, infinities and NaNs.  Prints the mismatch count.
#include <cstdio>
#include <cstring>
#include <vector>

#include "mac_internal.cuh"

using namespace mac;

namespace mac {
void set_last_cuda_error(cudaError_t, const char*, const char*, int) {}
}

__global__ void k_conv(const double* x, const float* f, unsigned* bad, long n) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float a = to_float_rn(x[i]), b = __double2float_rn(x[i]);
    const bool nan_a = a != a, nan_b = b != b;
    if (nan_a != nan_b || (!nan_a && __float_as_uint(a) != __float_as_uint(b))) atomicAdd(bad, 1u);
    const double c = to_double(f[i]), d = (double)f[i];
    const bool nan_c = c != c, nan_d = d != d;
    if (nan_c != nan_d ||
        (!nan_c && __double_as_longlong(c) != __double_as_longlong(d)))
        atomicAdd(bad + 1, 1u);
}

static unsigned long long rng_state = 0x9E3779B97F4A7C15ull;
static unsigned long long next64() {
    rng_state ^= rng_state << 13;
    rng_state ^= rng_state >> 7;
    rng_state ^= rng_state << 17;
    return rng_state;
}

int main() {
    std::vector<double> x;
    std::vector<float> f;
    const long nrand = 1 << 22;
    for (long i = 0; i < nrand; ++i) {
        unsigned long long u = next64();
        double v;
        std::memcpy(&v, &u, 8);
        x.push_back(v);
        unsigned w = (unsigned)next64();
        float g;
        std::memcpy(&g, &w, 4);
        f.push_back(g);
    }
    // doubles near the FP32 range and exactly at rounding ties
    for (int e = 880; e <= 1160; ++e)
        for (unsigned long long low : {0ull, 1ull, 0x0FFFFFFFull, 0x10000000ull, 0x10000001ull,
                                       0x1FFFFFFFull, 0x20000000ull, 0x30000000ull}) {
            for (unsigned long long top : {0ull, 1ull, 0x7FFFFFull, 0x400000ull}) {
                for (int sg = 0; sg < 2; ++sg) {
                    const unsigned long long u = ((unsigned long long)sg << 63) |
                                                 ((unsigned long long)e << 52) | (top << 29) | low;
                    double v;
                    std::memcpy(&v, &u, 8);
                    x.push_back(v);
                    f.push_back((float)(sg ? -1.0 : 1.0));
                }
            }
        }
    const double specials[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38,
                               1.1754943508222875e-38, 1.1754942106924411e-38, 1e-45, 1e300,
                               -1e300, 1.0 / 0.0, -1.0 / 0.0, 0.0 / 0.0};
    const float fspecial[] = {0.f, -0.f, 1e-45f, -1e-45f, 1.17549435e-38f, 3.40282347e38f,
                              1.0f / 0.0f, -1.0f / 0.0f, 0.0f / 0.0f, 1.5f, -2.25f};
    for (double v : specials) {
        x.push_back(v);
        f.push_back(1.0f);
    }
    for (float g : fspecial) {
        x.push_back(1.0);
        f.push_back(g);
    }
    const long n = (long)x.size();
    double* dx;
    float* df;
    unsigned* dbad;
    cudaMalloc(&dx, sizeof(double) * n);
    cudaMalloc(&df, sizeof(float) * n);
    cudaMalloc(&dbad, 2 * sizeof(unsigned));
    cudaMemcpy(dx, x.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(df, f.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemset(dbad, 0, 2 * sizeof(unsigned));
    k_conv<<<(unsigned)((n + 255) / 256), 256>>>(dx, df, dbad, n);
    unsigned bad[2] = {9, 9};
    cudaMemcpy(bad, dbad, sizeof(bad), cudaMemcpyDeviceToHost);
    const cudaError_t e = cudaGetLastError();
    printf("checked %ld mismatches_to_float %u mismatches_to_double %u status %s\n", n, bad[0],
           bad[1], cudaGetErrorString(e));
    return (e == cudaSuccess && bad[0] == 0 && bad[1] == 0) ? 0 : 1;
}
