// Checks recip_nr (mac_internal.cuh: reciprocal estimate + one third-order Newton step) against
// the IEEE FP64 division 1.0 / x: random doubles over the whole exponent range the function
// refines (biased exponents 64 .. 1980, both signs), every binade's end points and mantissas
// next to 1 and 2, and inputs outside that range (zero, subnormals, huge, infinities, NaN),
// which must take the division itself.  Prints the largest distance in units in the last place
// (ulp: difference of the bit patterns of two same-sign doubles), how many results differ from
// the division at all, and the fallback mismatches.
#include <cstdio>
#include <cstring>
#include <vector>

#include "mac_internal.cuh"

using namespace mac;

namespace mac {
void set_last_cuda_error(cudaError_t, const char*, const char*, int) {}
}

// out[0] = max ulp distance (refined range), out[1] = results != division (refined range),
// out[2] = fallback inputs whose result differs from the division (NaN == NaN)
__global__ void k_recip(const double* x, unsigned long long* out, long n) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    const double a = recip_nr(v), b = 1.0 / v;
    const unsigned ex = (unsigned)((unsigned long long)__double_as_longlong(v) >> 52) & 0x7FFu;
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    if (ex >= 64u && ex <= 1980u) {
        const long long d = ia > ib ? ia - ib : ib - ia;
        atomicMax(out, (unsigned long long)d);
        if (d != 0) atomicAdd(out + 1, 1ull);
    } else {
        const bool na = a != a, nb = b != b;
        if (na != nb || (!na && ia != ib)) atomicAdd(out + 2, 1ull);
    }
}

static unsigned long long rng_state = 0x2545F4914F6CDD1Dull;
static unsigned long long next64() {
    rng_state ^= rng_state << 13;
    rng_state ^= rng_state >> 7;
    rng_state ^= rng_state << 17;
    return rng_state;
}

static double from_bits(unsigned long long u) {
    double v;
    std::memcpy(&v, &u, 8);
    return v;
}

int main() {
    std::vector<double> x;
    const unsigned long long kMant = 0xFFFFFFFFFFFFFull;
    // random mantissas, uniformly random exponents in the refined range, both signs
    for (long i = 0; i < (1l << 23); ++i) {
        const unsigned long long r = next64();
        const unsigned long long e = 64ull + (next64() % (1980ull - 64ull + 1ull));
        x.push_back(from_bits((r & (1ull << 63)) | (e << 52) | (r & kMant)));
    }
    // every binade: its first and last mantissas and the ones next to them
    for (unsigned long long e = 64; e <= 1980; ++e)
        for (unsigned long long m : {0ull, 1ull, 2ull, kMant - 1ull, kMant, 0x8000000000000ull})
            for (int sg = 0; sg < 2; ++sg)
                x.push_back(from_bits(((unsigned long long)sg << 63) | (e << 52) | m));
    // outside the refined range: the division itself
    for (unsigned long long e : {0ull, 1ull, 30ull, 63ull, 1981ull, 2000ull, 2046ull})
        for (unsigned long long m : {0ull, 1ull, kMant, 0x123456789ABCDull})
            for (int sg = 0; sg < 2; ++sg)
                x.push_back(from_bits(((unsigned long long)sg << 63) | (e << 52) | m));
    x.push_back(from_bits(0x7FF0000000000000ull));   // +inf
    x.push_back(from_bits(0xFFF0000000000000ull));   // -inf
    x.push_back(from_bits(0x7FF8000000000000ull));   // NaN
    const long n = (long)x.size();
    double* dx;
    unsigned long long* dout;
    cudaMalloc(&dx, sizeof(double) * n);
    cudaMalloc(&dout, 3 * sizeof(unsigned long long));
    cudaMemcpy(dx, x.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemset(dout, 0, 3 * sizeof(unsigned long long));
    k_recip<<<(unsigned)((n + 255) / 256), 256>>>(dx, dout, n);
    unsigned long long out[3] = {~0ull, ~0ull, ~0ull};
    cudaMemcpy(out, dout, sizeof(out), cudaMemcpyDeviceToHost);
    const cudaError_t e = cudaGetLastError();
    printf("checked %ld max_ulp %llu differing %llu fallback_mismatches %llu status %s\n", n,
           out[0], out[1], out[2], cudaGetErrorString(e));
    cudaFree(dx);
    cudaFree(dout);
    return e == cudaSuccess ? 0 : 1;
}
