// Bottom solver of the multigrid (coarsest level, natural layout, FP64): device code shared by
// the bottom kernel (mac_kernels.cu) and the single-CTA tail V-cycle (mac_tail.cu).
// FBoxLib's default MAC bottom solve (Docs/mg/mg.tex:221-249): nub red/black Gauss-Seidel sweeps,
// BiCGStab to bottom_eps, nub sweeps; here BiCGStab is Jacobi preconditioned.
#pragma once

#include "mac_internal.cuh"

namespace mac {
namespace {

struct BotView {
    int n0, n1, n2, N;
    const double *bx, *by, *bz, *dg, *idg;
};

// Synchronisation policies of the bottom solver.  Sync128<NAMED>: 128 threads (four warps, so
// the four FP64 units of the SM share the work), work item p of a loop handled by warp p % 4
// (item permutation), reductions: xor-shuffle within each warp, then the four warp sums in a fixed
// order -- every thread gets the same value.  NAMED: barrier 1 over the first 128 threads of a
// larger CTA, else __syncthreads (a 128-thread CTA).  CtaSync: any CTA size, natural item order.
template <bool NAMED>
struct Sync128 {
    static __device__ __forceinline__ void sync() {
        if (NAMED)
            asm volatile("bar.sync 1, 128;" ::: "memory");
        else
            __syncthreads();
    }
    static __device__ __forceinline__ int tid() {
        const int t = threadIdx.x;
        return 4 * (t & 31) + (t >> 5);
    }
    static __device__ __forceinline__ int nt() { return 128; }
    static __device__ double sum(double v, double* sm) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
        sync();
        const double r = (sm[0] + sm[1]) + (sm[2] + sm[3]);
        sync();
        return r;
    }
    // two sums at once (one pair of barriers)
    static __device__ void sum2(double& a, double& b, double* sm) {
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if ((threadIdx.x & 31) == 0) {
            sm[threadIdx.x >> 5] = a;
            sm[4 + (threadIdx.x >> 5)] = b;
        }
        sync();
        a = (sm[0] + sm[1]) + (sm[2] + sm[3]);
        b = (sm[4] + sm[5]) + (sm[6] + sm[7]);
        sync();
    }
    // maximum of unsigned 64-bit keys (integer pipe)
    static __device__ unsigned long long umax(unsigned long long v, double* sm) {
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
            v = w > v ? w : v;
        }
        unsigned long long* u = reinterpret_cast<unsigned long long*>(sm);
        if ((threadIdx.x & 31) == 0) u[threadIdx.x >> 5] = v;
        sync();
        unsigned long long r = u[0];
        for (int w = 1; w < 4; ++w) r = u[w] > r ? u[w] : r;
        sync();
        return r;
    }
};

struct CtaSync {
    static __device__ __forceinline__ void sync() { __syncthreads(); }
    static __device__ __forceinline__ int tid() { return threadIdx.x; }
    static __device__ __forceinline__ int nt() { return blockDim.x; }
    static __device__ double sum(double v, double* sm) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if (lane == 0) sm[wid] = v;
        __syncthreads();
        if (wid == 0) {
            double r = lane < nw ? sm[lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
            if (lane == 0) sm[32] = r;
        }
        __syncthreads();
        const double r = sm[32];
        __syncthreads();
        return r;
    }
    static __device__ double max(double v, double* sm) {
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if (lane == 0) sm[wid] = v;
        __syncthreads();
        if (wid == 0) {
            double r = lane < nw ? sm[lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_down_sync(0xffffffffu, r, o));
            if (lane == 0) sm[32] = r;
        }
        __syncthreads();
        const double r = sm[32];
        __syncthreads();
        return r;
    }
    static __device__ void sum2(double& a, double& b, double* sm) {
        a = sum(a, sm);
        b = sum(b, sm);
    }
    static __device__ unsigned long long umax(unsigned long long v, double* sm) {
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
            v = w > v ? w : v;
        }
        unsigned long long* u = reinterpret_cast<unsigned long long*>(sm);
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if (lane == 0) u[wid] = v;
        __syncthreads();
        if (wid == 0) {
            unsigned long long r = lane < nw ? u[lane] : 0ull;
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long w = __shfl_down_sync(0xffffffffu, r, o);
                r = w > r ? w : r;
            }
            if (lane == 0) u[32] = r;
        }
        __syncthreads();
        const unsigned long long r = u[32];
        __syncthreads();
        return r;
    }
};

// |v| as an order-preserving integer key (the bit pattern of a non-negative double).
__device__ __forceinline__ unsigned long long abs_key(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ double key_value(unsigned long long k) {
    return __longlong_as_double((long long)k);
}

// Per-solve tables of the bottom operator (built by bot_prepare): for cell c and arm n (x-, x+,
// y-, y+, z-, z+) the neighbour index nb[n N + c] (periodic wrap; a wall arm has a zero
// coefficient) and gc[n N + c] = a_n(c) / diag(c), where A x = diag x - sum_n a_n x_n; the cell's
// colour (i + j + k) & 1 in nb[6 N + c].  With them a Gauss-Seidel update is
// x_c = f_c / diag_c + sum_n gc_n x_n (six FP64 fused multiply-adds) and A x = diag (x - sum_n
// gc_n x_n).  GB300 issues one FP64 warp instruction per about 64 cycles per SM sub-partition,
// whatever the number of active lanes, so the bottom is written to minimise FP64 instructions:
// integer index work is done once per solve, max-norms are taken on integer keys, and scalar
// divisions use recip_nr.
struct BotTables {
    int* nb;       // 7 N ints
    double* gc;    // 6 N doubles
    double* fi;    // N doubles: f / diag
};

template <class S>
__device__ void bot_prepare(const BotView& v, const BotTables& T) {
    const int N = v.N;
    for (int c = S::tid(); c < N; c += S::nt()) {
        const int i = c % v.n0;
        const int row = c / v.n0;
        const int j = row % v.n1;
        const int k = row / v.n1;
        const int im = i == 0 ? v.n0 - 1 : i - 1, ip = i == v.n0 - 1 ? 0 : i + 1;
        const int jm = j == 0 ? v.n1 - 1 : j - 1, jp = j == v.n1 - 1 ? 0 : j + 1;
        const int km = k == 0 ? v.n2 - 1 : k - 1, kp = k == v.n2 - 1 ? 0 : k + 1;
        const int cxm = im + v.n0 * (j + v.n1 * k), cxp = ip + v.n0 * (j + v.n1 * k);
        const int cym = i + v.n0 * (jm + v.n1 * k), cyp = i + v.n0 * (jp + v.n1 * k);
        const int czm = i + v.n0 * (j + v.n1 * km), czp = i + v.n0 * (j + v.n1 * kp);
        const double id = v.idg[c];
        T.nb[c] = cxm;
        T.nb[N + c] = cxp;
        T.nb[2 * N + c] = cym;
        T.nb[3 * N + c] = cyp;
        T.nb[4 * N + c] = czm;
        T.nb[5 * N + c] = czp;
        T.nb[6 * N + c] = (i + j + k) & 1;
        T.gc[c] = v.bx[c] * id;
        T.gc[N + c] = v.bx[cxp] * id;
        T.gc[2 * N + c] = v.by[c] * id;
        T.gc[3 * N + c] = v.by[cyp] * id;
        T.gc[4 * N + c] = v.bz[c] * id;
        T.gc[5 * N + c] = v.bz[czp] * id;
    }
    S::sync();
}

__device__ __forceinline__ double bot_gsum(const BotTables& T, int N, const double* __restrict__ x,
                                           int c, double s) {
#pragma unroll
    for (int n = 0; n < 6; ++n) s = fma(T.gc[n * N + c], x[T.nb[n * N + c]], s);
    return s;
}

// One red/black sweep.
template <class S>
__device__ __noinline__ void bot_gsrb(const BotView& v, const BotTables& T, double* x) {
    const int N = v.N;
    for (int colour = 0; colour < 2; ++colour) {
        for (int c = S::tid(); c < N; c += S::nt())
            if (T.nb[6 * N + c] == colour) x[c] = bot_gsum(T, N, x, c, T.fi[c]);
        S::sync();
    }
}

// y = A x
template <class S>
__device__ __noinline__ void bot_apply(const BotView& v, const BotTables& T, const double* x, double* y) {
    const int N = v.N;
    for (int c = S::tid(); c < N; c += S::nt()) {
        double t = x[c];
#pragma unroll
        for (int n = 0; n < 6; ++n) t = fma(-T.gc[n * N + c], x[T.nb[n * N + c]], t);
        y[c] = v.dg[c] * t;
    }
    S::sync();
}

// The bottom solve on FP64 arrays x (in/out) and f (in; mean removed here when singular):
// nub GS-RB sweeps, Jacobi-preconditioned BiCGStab reducing ||f - A x||_inf by eps, nub sweeps.
// scr holds kBotScrPerCell doubles per cell (14 N doubles, then 7 N ints).  Returns the BiCGStab
// iteration count.

template <class S>
__device__ int bottom_body(const BotView& v, double* x, double* f, double* scr, double* sm,
                           int singular, int nub, double eps, int max_iter) {
    const int N = v.N;
    const int tid = S::tid(), nt = S::nt();
    double* r = scr;
    double* rh = scr + N;
    double* p = scr + 2 * N;
    double* vv = scr + 3 * N;
    double* s = scr + 4 * N;
    double* t = scr + 5 * N;
    double* y = scr + 6 * N;
    BotTables T;
    T.gc = scr + 7 * N;
    T.fi = scr + 13 * N;
    T.nb = reinterpret_cast<int*>(scr + 14 * N);
    bot_prepare<S>(v, T);
    double loc = 0.0;
    for (int c = tid; c < N; c += nt) loc += f[c];
    const double mean = S::sum(loc, sm) / N;
    for (int c = tid; c < N; c += nt) {
        if (singular) f[c] -= mean;
        T.fi[c] = f[c] * v.idg[c];
    }
    S::sync();
    for (int it = 0; it < nub; ++it) bot_gsrb<S>(v, T, x);
    bot_apply<S>(v, T, x, t);
    unsigned long long kmax = 0;
    loc = 0.0;
    for (int c = tid; c < N; c += nt) {
        const double rc = f[c] - t[c];
        r[c] = rc;
        rh[c] = rc;
        p[c] = 0.0;
        vv[c] = 0.0;
        const unsigned long long key = abs_key(rc);
        kmax = key > kmax ? key : kmax;
        loc = fma(rc, rc, loc);
    }
    const double r0 = key_value(S::umax(kmax, sm));
    double rho = S::sum(loc, sm);   // (rh, r) of the first iteration
    int count = 0;
    if (r0 > 0.0) {
        const double tol = eps * r0;
        double rho_old = 1.0, alpha = 1.0, omega = 1.0;
        for (int it = 0; it < max_iter; ++it) {
            ++count;
            if (rho == 0.0) break;
            const double beta = (rho * alpha) * recip_nr(rho_old * omega);
            for (int c = tid; c < N; c += nt) {
                const double pc = fma(beta, fma(-omega, vv[c], p[c]), r[c]);
                p[c] = pc;
                y[c] = pc * v.idg[c];
            }
            S::sync();
            bot_apply<S>(v, T, y, vv);
            loc = 0.0;
            for (int c = tid; c < N; c += nt) loc = fma(rh[c], vv[c], loc);
            const double rv = S::sum(loc, sm);
            if (rv == 0.0) break;
            alpha = rho * recip_nr(rv);
            kmax = 0;
            for (int c = tid; c < N; c += nt) {
                const double sc = fma(-alpha, vv[c], r[c]);
                s[c] = sc;
                x[c] = fma(alpha, y[c], x[c]);
                const unsigned long long key = abs_key(sc);
                kmax = key > kmax ? key : kmax;
            }
            const double sn = key_value(S::umax(kmax, sm));
            if (sn <= tol) break;
            for (int c = tid; c < N; c += nt) y[c] = s[c] * v.idg[c];
            S::sync();
            bot_apply<S>(v, T, y, t);
            double l1 = 0.0, l2 = 0.0;
            for (int c = tid; c < N; c += nt) {
                l1 = fma(t[c], s[c], l1);
                l2 = fma(t[c], t[c], l2);
            }
            S::sum2(l1, l2, sm);
            omega = l2 > 0.0 ? l1 * recip_nr(l2) : 0.0;
            kmax = 0;
            loc = 0.0;
            for (int c = tid; c < N; c += nt) {
                x[c] = fma(omega, y[c], x[c]);
                const double rc = fma(-omega, t[c], s[c]);
                r[c] = rc;
                const unsigned long long key = abs_key(rc);
                kmax = key > kmax ? key : kmax;
                loc = fma(rh[c], rc, loc);
            }
            const double rn = key_value(S::umax(kmax, sm));
            rho_old = rho;
            rho = S::sum(loc, sm);
            if (rn <= tol || omega == 0.0) break;
        }
    }
    S::sync();
    for (int it = 0; it < nub; ++it) bot_gsrb<S>(v, T, x);
    return count;
}


}  // namespace
}  // namespace mac
