// Flexible conjugate gradients (one previous direction kept) around the FP32 V-cycle, inside a
// mixed-precision refinement step.  With r the FP32 right-hand side of the step (the FP64
// residual rounded) and z = V(r) one V-cycle from z = 0:
//
//   w = L z;  beta = (z, q')/(p', q');  p = z - beta p';  q = w - beta q'
//   alpha = (p, r)/(p, q);  x += alpha p;  r -= alpha q
//
// and the step ends with phi += x in FP64.  The V-cycle ends with a half-sweep of colour 1, after
// which (L z) = r on every colour-1 cell, so only the colour-0 half of w is computed (and stored).
// The inner products are expanded so that one pass gives all of them:
//   (p, q) = (z, w) - beta (z, q') - beta (p', w) + beta^2 (p', q'),   (p, r) = (z, r) - beta (p', r)
// Every product is taken in FP32 per thread and summed in FP64 over the grid in a fixed order
// (per-block partials, then the last block to finish adds them up and forms alpha and beta), so
// the result is the same from run to run.  The V-cycle itself is unchanged (the multigrid of
// Source/mac_multigrid.f90:56-67); this only chooses how its corrections are combined.
#include "mac_internal.cuh"
#include "mac_otf.cuh"

namespace mac {
namespace {

constexpr int kKB = 128;        // threads of the inner-product kernel
constexpr int kKPlanes = 32;    // planes per block of the inner-product kernel
constexpr int kKDots = 5;       // (z,w) (z,r) (z,q') (p',w) (p',r)
constexpr int kUB = 256;        // threads of the elementwise kernels

__device__ __forceinline__ float wsum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double wsumd(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// w = L z on the colour-0 cells (w0, when non-null, receives it) and the five inner products.
// OTF: coefficients from rho32 (otf_cell); else the stored FP32 level-0 operator.
template <int DM, bool OTF, bool FIRST>
__global__ void __launch_bounds__(kKB)
k_fcg_dots(Dims F, OtfParams P, LevelArrays<float> A, const float* __restrict__ z,
           const float* __restrict__ r, const float* __restrict__ p, const float* __restrict__ q,
           float* __restrict__ w0, double* __restrict__ partial, double* __restrict__ sc,
           unsigned* __restrict__ count) {
    pdl_wait();
    pdl_trigger();
    __shared__ double sred[kKB / 32][kKDots];
    __shared__ int s_last;
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k0 = blockIdx.z * kKPlanes;
    const long half = F.half;
    float zw = 0.f, zr = 0.f, zq = 0.f, pw = 0.f, pr = 0.f;
    if (h < F.hn0 && j < F.n1) {
        for (int k = k0; k < k0 + kKPlanes && k < F.n2; ++k) {
            const int me = (j + F.n1 * k) * F.hn0 + h;
            const int i = 2 * h + ((j + k) & 1);
            Nb nb;
            nbrs(F, 0, h, j, k, nb);
            float acc = 0.f, diag;
            if (OTF) {
                otf_cell<DM>(P, nb, i, j, k, P.rho[me], P.rho + half, z + half, acc, diag);
            } else {
                const float* zo = z + half;
                acc = fmaf(A.bx[me], zo[nb.xm], acc);
                acc = fmaf(A.bx[half + nb.xp], zo[nb.xp], acc);
                acc = fmaf(A.by[me], zo[nb.ym], acc);
                acc = fmaf(A.by[half + nb.yp], zo[nb.yp], acc);
                acc = fmaf(A.bz[me], zo[nb.zm], acc);
                acc = fmaf(A.bz[half + nb.zp], zo[nb.zp], acc);
                diag = A.diag[me];
            }
            const float z0 = z[me], z1 = z[half + me];
            const float r0 = r[me], r1 = r[half + me];
            const float w = fmaf(diag, z0, -acc);
            if (w0) w0[me] = w;
            zw = fmaf(z0, w, fmaf(z1, r1, zw));
            zr = fmaf(z0, r0, fmaf(z1, r1, zr));
            if (!FIRST) {
                const float p0 = p[me], p1 = p[half + me];
                const float q0 = q[me], q1 = q[half + me];
                zq = fmaf(z0, q0, fmaf(z1, q1, zq));
                pw = fmaf(p0, w, fmaf(p1, r1, pw));
                pr = fmaf(p0, r0, fmaf(p1, r1, pr));
            }
        }
    }
    const int t = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = t & 31, wid = t >> 5;
    float v[kKDots] = {zw, zr, zq, pw, pr};
#pragma unroll
    for (int a = 0; a < kKDots; ++a) v[a] = wsum(v[a]);
    if (lane == 0)
#pragma unroll
        for (int a = 0; a < kKDots; ++a) sred[wid][a] = to_double(v[a]);
    __syncthreads();
    const int nblk = gridDim.x * gridDim.y * gridDim.z;
    const int blk = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    if (t == 0) {
        for (int a = 0; a < kKDots; ++a) {
            double s = 0.0;
            for (int w = 0; w < kKB / 32; ++w) s += sred[w][a];
            partial[(size_t)kKDots * blk + a] = s;
        }
        __threadfence();
        s_last = atomicAdd(count, 1u) == (unsigned)(nblk - 1);
    }
    __syncthreads();
    if (!s_last) return;
    // the last block: fixed-order sums over the block partials, then alpha and beta
    __threadfence();
    double s[kKDots] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = t; b < nblk; b += kKB)
#pragma unroll
        for (int a = 0; a < kKDots; ++a) s[a] += __ldcg(partial + (size_t)kKDots * b + a);
#pragma unroll
    for (int a = 0; a < kKDots; ++a) s[a] = wsumd(s[a]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int a = 0; a < kKDots; ++a) sred[wid][a] = s[a];
    __syncthreads();
    if (t == 0) {
        double d[kKDots];
        for (int a = 0; a < kKDots; ++a) {
            d[a] = 0.0;
            for (int w = 0; w < kKB / 32; ++w) d[a] += sred[w][a];
        }
        const double dzw = d[0], dzr = d[1], dzq = d[2], dpw = d[3], dpr = d[4];
        double beta = 0.0, pq = dzw, prr = dzr;
        if (!FIRST) {
            const double pq_prev = sc[2];
            beta = pq_prev > 0.0 ? dzq / pq_prev : 0.0;
            pq = dzw - beta * dzq - beta * dpw + beta * beta * pq_prev;
            prr = dzr - beta * dpr;
        }
        double alpha = prr / pq;
        if (!(pq > 0.0) || !isfinite(alpha) || !isfinite(beta)) {
            // no usable step length: take the plain V-cycle correction (p = z, alpha = 1)
            beta = 0.0;
            alpha = 1.0;
            pq = dzw > 0.0 ? dzw : 1.0;
        }
        sc[0] = alpha;
        sc[1] = beta;
        sc[2] = pq;
        *count = 0u;
    }
}

// p = z - beta p', q = w - beta q', x += alpha p, r -= alpha q, and z = 0 for the next V-cycle
// (FIRST: p = z, q = w, x = alpha z).  V = 4: float4 groups (half % 4 == 0), else single cells.
template <bool FIRST, int V>
__global__ void __launch_bounds__(kUB)
k_fcg_update(long n, long half, float* __restrict__ z, float* __restrict__ r,
             const float* __restrict__ w0, float* __restrict__ p, float* __restrict__ q,
             float* __restrict__ x, const double* __restrict__ sc) {
    pdl_wait();
    pdl_trigger();
    const long g = (blockIdx.x * (long)blockDim.x + threadIdx.x) * V;
    if (g >= n) return;
    const float a = to_float_rn(sc[0]), b = to_float_rn(sc[1]);
    if (V == 4) {
        const float4 zv = *reinterpret_cast<const float4*>(z + g);
        const float4 rv = *reinterpret_cast<const float4*>(r + g);
        const float4 wv = g < half ? *reinterpret_cast<const float4*>(w0 + g) : rv;
        float4 pn, qn, xn;
        if (FIRST) {
            pn = zv;
            qn = wv;
            xn = make_float4(a * zv.x, a * zv.y, a * zv.z, a * zv.w);
        } else {
            const float4 pv = *reinterpret_cast<const float4*>(p + g);
            const float4 qv = *reinterpret_cast<const float4*>(q + g);
            const float4 xv = *reinterpret_cast<const float4*>(x + g);
            pn = make_float4(fmaf(-b, pv.x, zv.x), fmaf(-b, pv.y, zv.y), fmaf(-b, pv.z, zv.z),
                             fmaf(-b, pv.w, zv.w));
            qn = make_float4(fmaf(-b, qv.x, wv.x), fmaf(-b, qv.y, wv.y), fmaf(-b, qv.z, wv.z),
                             fmaf(-b, qv.w, wv.w));
            xn = make_float4(fmaf(a, pn.x, xv.x), fmaf(a, pn.y, xv.y), fmaf(a, pn.z, xv.z),
                             fmaf(a, pn.w, xv.w));
        }
        const float4 rn = make_float4(fmaf(-a, qn.x, rv.x), fmaf(-a, qn.y, rv.y),
                                      fmaf(-a, qn.z, rv.z), fmaf(-a, qn.w, rv.w));
        *reinterpret_cast<float4*>(p + g) = pn;
        *reinterpret_cast<float4*>(q + g) = qn;
        *reinterpret_cast<float4*>(x + g) = xn;
        *reinterpret_cast<float4*>(r + g) = rn;
        *reinterpret_cast<float4*>(z + g) = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        const float zv = z[g], rv = r[g];
        const float wv = g < half ? w0[g] : rv;
        float pn, qn, xn;
        if (FIRST) {
            pn = zv;
            qn = wv;
            xn = a * zv;
        } else {
            pn = fmaf(-b, p[g], zv);
            qn = fmaf(-b, q[g], wv);
            xn = fmaf(a, pn, x[g]);
        }
        p[g] = pn;
        q[g] = qn;
        x[g] = xn;
        r[g] = fmaf(-a, qn, rv);
        z[g] = 0.f;
    }
}

// Last inner step: phi += x + alpha (z - beta p') in FP64 (FIRST: phi += alpha z).
template <bool FIRST>
__global__ void __launch_bounds__(kUB)
k_fcg_final(long n, double* __restrict__ phi, const float* __restrict__ z,
            const float* __restrict__ p, const float* __restrict__ x,
            const double* __restrict__ sc) {
    pdl_wait();
    pdl_trigger();
    const long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (g >= n) return;
    const float a = to_float_rn(sc[0]);
    float e;
    if (FIRST) {
        e = a * z[g];
    } else {
        const float b = to_float_rn(sc[1]);
        e = fmaf(a, fmaf(-b, p[g], z[g]), x[g]);
    }
    phi[g] += to_double(e);
}

template <int DM, bool OTF>
void dots_dm_otf(const Dims& d, const OtfParams& P, const LevelArrays<float>& A, bool first,
                 const KrylovBufs& K, bool store_w, cudaStream_t s) {
    Grid3 g = grid3(d.hn0, d.n1, 1);
    g.grid.z = ceil_div(d.n2, kKPlanes);
    float* w0 = store_w ? K.w0 : nullptr;
    if (first)
        launch_chain(k_fcg_dots<DM, OTF, true>, g.grid, g.block, 0, s, d, P, A,
                     (const float*)A.phi, (const float*)A.f, (const float*)K.p,
                     (const float*)K.q, w0, K.partial, K.scalars, K.count);
    else
        launch_chain(k_fcg_dots<DM, OTF, false>, g.grid, g.block, 0, s, d, P, A,
                     (const float*)A.phi, (const float*)A.f, (const float*)K.p,
                     (const float*)K.q, w0, K.partial, K.scalars, K.count);
}

}  // namespace

int krylov_partials(const Dims& d) {
    Grid3 g = grid3(d.hn0, d.n1, 1);
    g.grid.z = ceil_div(d.n2, kKPlanes);
    return (int)(g.grid.x * g.grid.y * g.grid.z) * kKDots;
}

void launch_fcg_dots(const Dims& d, int dm, bool otf, const OtfParams& P,
                     const LevelArrays<float>& A, const KrylovBufs& K, bool first, bool store_w,
                     cudaStream_t s) {
    // (the OTF parameters are only read when otf is set; the stored operator only when not)
    if (dm == 3) {
        if (otf)
            dots_dm_otf<3, true>(d, P, A, first, K, store_w, s);
        else
            dots_dm_otf<3, false>(d, P, A, first, K, store_w, s);
    } else {
        if (otf)
            dots_dm_otf<2, true>(d, P, A, first, K, store_w, s);
        else
            dots_dm_otf<2, false>(d, P, A, first, K, store_w, s);
    }
}

void launch_fcg_update(const Dims& d, const LevelArrays<float>& A, const KrylovBufs& K,
                       bool first, cudaStream_t s) {
    const long n = d.ncell, half = d.half;
    float* z = A.phi;
    float* r = A.f;
    if (half % 4 == 0) {
        const int nb = ceil_div(n / 4, kUB);
        if (first)
            launch_chain(k_fcg_update<true, 4>, dim3(nb), dim3(kUB), 0, s, n, half, z, r,
                         (const float*)K.w0, K.p, K.q, K.x, (const double*)K.scalars);
        else
            launch_chain(k_fcg_update<false, 4>, dim3(nb), dim3(kUB), 0, s, n, half, z, r,
                         (const float*)K.w0, K.p, K.q, K.x, (const double*)K.scalars);
    } else {
        const int nb = ceil_div(n, kUB);
        if (first)
            launch_chain(k_fcg_update<true, 1>, dim3(nb), dim3(kUB), 0, s, n, half, z, r,
                         (const float*)K.w0, K.p, K.q, K.x, (const double*)K.scalars);
        else
            launch_chain(k_fcg_update<false, 1>, dim3(nb), dim3(kUB), 0, s, n, half, z, r,
                         (const float*)K.w0, K.p, K.q, K.x, (const double*)K.scalars);
    }
}

void launch_fcg_final(const Dims& d, double* phi, const LevelArrays<float>& A,
                      const KrylovBufs& K, bool first, cudaStream_t s) {
    const long n = d.ncell;
    const int nb = ceil_div(n, kUB);
    if (first)
        launch_chain(k_fcg_final<true>, dim3(nb), dim3(kUB), 0, s, n, phi, (const float*)A.phi,
                     (const float*)K.p, (const float*)K.x, (const double*)K.scalars);
    else
        launch_chain(k_fcg_final<false>, dim3(nb), dim3(kUB), 0, s, n, phi, (const float*)A.phi,
                     (const float*)K.p, (const float*)K.x, (const double*)K.scalars);
}

}  // namespace mac
