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

__device__ __forceinline__ double bot_arms(const BotView& v, const double* __restrict__ x, int c) {
    const int i = c % v.n0;
    const int row = c / v.n0;
    const int j = row % v.n1;
    const int k = row / v.n1;
    const int im = i == 0 ? v.n0 - 1 : i - 1, ip = i == v.n0 - 1 ? 0 : i + 1;
    const int jm = j == 0 ? v.n1 - 1 : j - 1, jp = j == v.n1 - 1 ? 0 : j + 1;
    const int km = k == 0 ? v.n2 - 1 : k - 1, kp = k == v.n2 - 1 ? 0 : k + 1;
    const int cxp = ip + v.n0 * (j + v.n1 * k), cxm = im + v.n0 * (j + v.n1 * k);
    const int cyp = i + v.n0 * (jp + v.n1 * k), cym = i + v.n0 * (jm + v.n1 * k);
    const int czp = i + v.n0 * (j + v.n1 * kp), czm = i + v.n0 * (j + v.n1 * km);
    double s = v.bx[c] * x[cxm];
    s = fma(v.bx[cxp], x[cxp], s);
    s = fma(v.by[c], x[cym], s);
    s = fma(v.by[cyp], x[cyp], s);
    s = fma(v.bz[c], x[czm], s);
    s = fma(v.bz[czp], x[czp], s);
    return s;
}

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
    static __device__ double max(double v, double* sm) {
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
        sync();
        const double r = fmax(fmax(sm[0], sm[1]), fmax(sm[2], sm[3]));
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
};

// One red/black sweep.  With an even x extent the cells of a colour are enumerated directly
// (cell p of the colour: h = p % (n0/2), row = p / (n0/2), i = 2h + (colour + j + k) & 1).
template <class S>
__device__ void bot_gsrb(const BotView& v, double* x, const double* f) {
    const bool even = (v.n0 & 1) == 0;
    const int hn0 = v.n0 >> 1;
    for (int colour = 0; colour < 2; ++colour) {
        if (even) {
            const int nc = v.N >> 1;
            for (int p = S::tid(); p < nc; p += S::nt()) {
                const int h = p % hn0, row = p / hn0, j = row % v.n1, k = row / v.n1;
                const int c = 2 * h + ((colour + j + k) & 1) + v.n0 * row;
                x[c] = (f[c] + bot_arms(v, x, c)) * v.idg[c];
            }
        } else {
            for (int c = S::tid(); c < v.N; c += S::nt()) {
                const int i = c % v.n0, row = c / v.n0, j = row % v.n1, k = row / v.n1;
                if (((i + j + k) & 1) != colour) continue;
                x[c] = (f[c] + bot_arms(v, x, c)) * v.idg[c];
            }
        }
        S::sync();
    }
}

template <class S>
__device__ void bot_apply(const BotView& v, const double* x, double* y) {
    for (int c = S::tid(); c < v.N; c += S::nt()) y[c] = v.dg[c] * x[c] - bot_arms(v, x, c);
    S::sync();
}

// The bottom solve on FP64 arrays x (in/out) and f (in; mean removed here when singular):
// nub GS-RB sweeps, Jacobi-preconditioned BiCGStab reducing ||f - A x||_inf by eps, nub sweeps.
// scr holds 7 N doubles.  Returns the BiCGStab iteration count.
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
    double loc = 0.0;
    for (int c = tid; c < N; c += nt) loc += f[c];
    const double mean = S::sum(loc, sm) / N;
    if (singular)
        for (int c = tid; c < N; c += nt) f[c] -= mean;
    S::sync();
    for (int it = 0; it < nub; ++it) bot_gsrb<S>(v, x, f);
    bot_apply<S>(v, x, t);
    loc = 0.0;
    for (int c = tid; c < N; c += nt) {
        r[c] = f[c] - t[c];
        rh[c] = r[c];
        p[c] = 0.0;
        vv[c] = 0.0;
        loc = fmax(loc, fabs(r[c]));
    }
    const double r0 = S::max(loc, sm);
    int count = 0;
    if (r0 > 0.0) {
        const double tol = eps * r0;
        double rho_old = 1.0, alpha = 1.0, omega = 1.0;
        for (int it = 0; it < max_iter; ++it) {
            ++count;
            loc = 0.0;
            for (int c = tid; c < N; c += nt) loc += rh[c] * r[c];
            const double rho = S::sum(loc, sm);
            if (rho == 0.0) break;
            const double beta = (rho / rho_old) * (alpha / omega);
            for (int c = tid; c < N; c += nt) {
                p[c] = r[c] + beta * (p[c] - omega * vv[c]);
                y[c] = p[c] * v.idg[c];
            }
            S::sync();
            bot_apply<S>(v, y, vv);
            loc = 0.0;
            for (int c = tid; c < N; c += nt) loc += rh[c] * vv[c];
            const double rv = S::sum(loc, sm);
            if (rv == 0.0) break;
            alpha = rho / rv;
            loc = 0.0;
            for (int c = tid; c < N; c += nt) {
                s[c] = r[c] - alpha * vv[c];
                loc = fmax(loc, fabs(s[c]));
            }
            const double sn = S::max(loc, sm);
            if (sn <= tol) {
                for (int c = tid; c < N; c += nt) x[c] += alpha * y[c];
                S::sync();
                break;
            }
            for (int c = tid; c < N; c += nt) x[c] += alpha * y[c];
            for (int c = tid; c < N; c += nt) y[c] = s[c] * v.idg[c];
            S::sync();
            bot_apply<S>(v, y, t);
            double l1 = 0.0, l2 = 0.0;
            for (int c = tid; c < N; c += nt) {
                l1 += t[c] * s[c];
                l2 += t[c] * t[c];
            }
            const double ts = S::sum(l1, sm);
            const double tt = S::sum(l2, sm);
            omega = tt > 0.0 ? ts / tt : 0.0;
            loc = 0.0;
            for (int c = tid; c < N; c += nt) {
                x[c] += omega * y[c];
                r[c] = s[c] - omega * t[c];
                loc = fmax(loc, fabs(r[c]));
            }
            const double rn = S::max(loc, sm);
            if (rn <= tol || omega == 0.0) break;
            rho_old = rho;
        }
    }
    for (int it = 0; it < nub; ++it) bot_gsrb<S>(v, x, f);
    return count;
}


}  // namespace
}  // namespace mac
