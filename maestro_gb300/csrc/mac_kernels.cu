// Multigrid kernels of the GB300 MAC projection: red/black Gauss-Seidel, defect + restriction,
// prolongation, residual norms and the single-CTA FP64 BiCGStab bottom solver.
//
// Arithmetic follows the FBoxLib cell-centred MG as described in MAESTRO's Docs/mg/mg.tex
// (:196-211 smoothers, :221-259 bottom solvers, :325-375 V-cycle flow); the level layout and
// the boundary trick are described in mac_internal.cuh.
#include "mac_internal.cuh"

namespace mac {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }

// Neighbour offsets (relative to the other colour's half) of split-layout cell (h, j, k) of
// colour `colour`.  x-neighbours of cell i = 2h + s are at h-1+s and h+s; y/z-neighbours keep h.
struct Nbr {
    int xm, xp, ym, yp, zm, zp;
};

__device__ __forceinline__ void split_nbrs(const Dims& d, int colour, int h, int j, int k, Nbr& nb) {
    const int s = (colour + j + k) & 1;
    int hm = h - 1 + s;
    hm += (hm < 0) ? d.hn0 : 0;
    int hp = h + s;
    hp -= (hp >= d.hn0) ? d.hn0 : 0;
    const int jm = (j == 0) ? d.n1 - 1 : j - 1;
    const int jp = (j == d.n1 - 1) ? 0 : j + 1;
    const int km = (k == 0) ? d.n2 - 1 : k - 1;
    const int kp = (k == d.n2 - 1) ? 0 : k + 1;
    const int row = (j + d.n1 * k) * d.hn0;
    nb.xm = row + hm;
    nb.xp = row + hp;
    nb.ym = (jm + d.n1 * k) * d.hn0 + h;
    nb.yp = (jp + d.n1 * k) * d.hn0 + h;
    nb.zm = (j + d.n1 * km) * d.hn0 + h;
    nb.zp = (j + d.n1 * kp) * d.hn0 + h;
}

// acc + sum over the six arms of beta'_face * u_neighbour for a split-layout cell.
// own = pointers to the cell's colour half, oth = the other colour's half.
template <typename T>
__device__ __forceinline__ T arms(T acc, int me, const Nbr& nb, const T* __restrict__ uo,
                                  const T* __restrict__ bxs, const T* __restrict__ bys,
                                  const T* __restrict__ bzs, const T* __restrict__ bxo,
                                  const T* __restrict__ byo, const T* __restrict__ bzo) {
    acc = fmaT(bxs[me], uo[nb.xm], acc);
    acc = fmaT(bxo[nb.xp], uo[nb.xp], acc);
    acc = fmaT(bys[me], uo[nb.ym], acc);
    acc = fmaT(byo[nb.yp], uo[nb.yp], acc);
    acc = fmaT(bzs[me], uo[nb.zm], acc);
    acc = fmaT(bzo[nb.zp], uo[nb.zp], acc);
    return acc;
}

__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(fabs(v));
}

__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long v) {
    __shared__ unsigned long long sm[32];
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = (lane < (int)(blockDim.x >> 5)) ? sm[lane] : 0ull;
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
            v = w > v ? w : v;
        }
    }
    return v;
}

// ---- red/black Gauss-Seidel half sweep (one colour) -----------------------------------------
template <typename T>
__global__ void __launch_bounds__(kBlock)
k_gsrb(Dims d, int colour, T* __restrict__ us, const T* __restrict__ uo, const T* __restrict__ fs,
       const T* __restrict__ bxs, const T* __restrict__ bys, const T* __restrict__ bzs,
       const T* __restrict__ bxo, const T* __restrict__ byo, const T* __restrict__ bzo,
       const T* __restrict__ ids) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d.half) return;
    const int h = q % d.hn0;
    const int row = q / d.hn0;
    const int j = row % d.n1;
    const int k = row / d.n1;
    Nbr nb;
    split_nbrs(d, colour, h, j, k, nb);
    T acc = arms<T>(fs[q], q, nb, uo, bxs, bys, bzs, bxo, byo, bzo);
    us[q] = acc * ids[q];
}

// ---- defect r = f - L u on the children of each coarse cell, averaged into the coarse rhs ---
template <typename T, bool RED_ONLY>
__global__ void __launch_bounds__(kBlock)
k_resid_restrict(Dims F, Dims C, const T* __restrict__ u, const T* __restrict__ f,
                 const T* __restrict__ bx, const T* __restrict__ by, const T* __restrict__ bz,
                 const T* __restrict__ dg, T* __restrict__ fc) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= C.ncell) return;
    const int I = q % C.n0;
    const int row = q / C.n0;
    const int J = row % C.n1;
    const int K = row / C.n1;
    T sum = T(0);
    for (int b = 0; b < F.rz; ++b) {
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            const int j = 2 * J + a;
            const int k = F.rz == 2 ? 2 * K + b : K;
#pragma unroll
            for (int colour = 0; colour < (RED_ONLY ? 1 : 2); ++colour) {
                const int off = colour * F.half, oth = (colour ^ 1) * F.half;
                Nbr nb;
                split_nbrs(F, colour, I, j, k, nb);
                const int me = (j + F.n1 * k) * F.hn0 + I;
                T r = fmaT(-dg[off + me], u[off + me], f[off + me]);
                r = arms<T>(r, me, nb, u + oth, bx + off, by + off, bz + off, bx + oth, by + oth,
                            bz + oth);
                sum += r;
            }
        }
    }
    int ci;
    if (C.split)
        ci = ((I + J + K) & 1) * C.half + (J + C.n1 * K) * C.hn0 + (I >> 1);
    else
        ci = I + C.n0 * (J + C.n1 * K);
    fc[ci] = sum * (T)(1.0 / (4 * F.rz));
}

// ---- prolongation: u_fine += (bi/tri)linear interpolation of the coarse correction ----------
__device__ __forceinline__ int ghost_fix(int q, int n, int blo, int bhi, float& sgn) {
    if (q < 0) {
        if (blo == MAC_BC_PER) return n - 1;
        sgn = (blo == MAC_BC_DIR) ? -1.f : 1.f;
        return 0;
    }
    if (q >= n) {
        if (bhi == MAC_BC_PER) return 0;
        sgn = (bhi == MAC_BC_DIR) ? -1.f : 1.f;
        return n - 1;
    }
    return q;
}

template <typename T>
__global__ void __launch_bounds__(kBlock)
k_prolong_add(Dims F, Dims C, BcDesc bc, const T* __restrict__ ec, T* __restrict__ u) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= F.half) return;
    const int h = q % F.hn0;
    const int row = q / F.hn0;
    const int j = row % F.n1;
    const int k = row / F.n1;
    const int I = h;
    const int J = j >> 1;
    const int oj = (j & 1) ? 1 : -1;
    int K, ok;
    if (F.rz == 2) {
        K = k >> 1;
        ok = (k & 1) ? 1 : -1;
    } else {
        K = k;
        ok = 0;
    }
    float sJ = 1.f, sK = 1.f, sIm = 1.f, sIp = 1.f;
    const int J2 = ghost_fix(J + oj, C.n1, bc.lo[1], bc.hi[1], sJ);
    const int K2 = ok ? ghost_fix(K + ok, C.n2, bc.lo[2], bc.hi[2], sK) : K;
    const int Im = ghost_fix(I - 1, C.n0, bc.lo[0], bc.hi[0], sIm);
    const int Ip = ghost_fix(I + 1, C.n0, bc.lo[0], bc.hi[0], sIp);
    const T wz0 = ok ? T(0.75) : T(1), wz1 = ok ? T(0.25) : T(0);
    auto cval = [&](int X, int Y, int Z) -> T {
        int ci;
        if (C.split)
            ci = ((X + Y + Z) & 1) * C.half + (Y + C.n1 * Z) * C.hn0 + (X >> 1);
        else
            ci = X + C.n0 * (Y + C.n1 * Z);
        return ec[ci];
    };
    auto col = [&](int X) -> T {
        T a = T(0.75) * cval(X, J, K) + T(0.25) * (T)sJ * cval(X, J2, K);
        T v = wz0 * a;
        if (ok) {
            T b = T(0.75) * cval(X, J, K2) + T(0.25) * (T)sJ * cval(X, J2, K2);
            v += wz1 * (T)sK * b;
        }
        return v;
    };
    const T vI = col(I), vm = col(Im), vp = col(Ip);
    const int cA = (j + k) & 1;   // colour of fine cell 2h
    const int idx = row * F.hn0 + h;
    u[cA * F.half + idx] += T(0.75) * vI + T(0.25) * (T)sIm * vm;
    u[(cA ^ 1) * F.half + idx] += T(0.75) * vI + T(0.25) * (T)sIp * vp;
}

// ---- residual max-norm (FP64 accumulation of |r|) ---------------------------------------------
template <typename T, bool RED_ONLY>
__global__ void __launch_bounds__(kBlock)
k_resid_norm(Dims F, const T* __restrict__ u, const T* __restrict__ f, const T* __restrict__ bx,
             const T* __restrict__ by, const T* __restrict__ bz, const T* __restrict__ dg,
             unsigned long long* __restrict__ maxbits) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long m = 0ull;
    if (q < F.half) {
        const int h = q % F.hn0;
        const int row = q / F.hn0;
        const int j = row % F.n1;
        const int k = row / F.n1;
#pragma unroll
        for (int colour = 0; colour < (RED_ONLY ? 1 : 2); ++colour) {
            const int off = colour * F.half, oth = (colour ^ 1) * F.half;
            Nbr nb;
            split_nbrs(F, colour, h, j, k, nb);
            T r = fmaT(-dg[off + q], u[off + q], f[off + q]);
            r = arms<T>(r, q, nb, u + oth, bx + off, by + off, bz + off, bx + oth, by + oth,
                        bz + oth);
            const unsigned long long b = abs_bits((double)r);
            m = b > m ? b : m;
        }
    }
    m = block_max_u64(m);
    if (threadIdx.x == 0 && m) atomicMax(maxbits, m);
}

// FP64 residual of the whole fine level, stored as FP32 (the refinement right-hand side).
__global__ void __launch_bounds__(kBlock)
k_resid64_to32(Dims F, const double* __restrict__ u, const double* __restrict__ f,
               const double* __restrict__ bx, const double* __restrict__ by,
               const double* __restrict__ bz, const double* __restrict__ dg,
               float* __restrict__ r32, unsigned long long* __restrict__ maxbits) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long m = 0ull;
    if (q < F.half) {
        const int h = q % F.hn0;
        const int row = q / F.hn0;
        const int j = row % F.n1;
        const int k = row / F.n1;
#pragma unroll
        for (int colour = 0; colour < 2; ++colour) {
            const int off = colour * F.half, oth = (colour ^ 1) * F.half;
            Nbr nb;
            split_nbrs(F, colour, h, j, k, nb);
            double r = fma(-dg[off + q], u[off + q], f[off + q]);
            r = arms<double>(r, q, nb, u + oth, bx + off, by + off, bz + off, bx + oth, by + oth,
                             bz + oth);
            r32[off + q] = (float)r;
            const unsigned long long b = abs_bits(r);
            m = b > m ? b : m;
        }
    }
    m = block_max_u64(m);
    if (threadIdx.x == 0 && m) atomicMax(maxbits, m);
}

__global__ void __launch_bounds__(kBlock)
k_accumulate(int n, double* __restrict__ u, const float* __restrict__ e) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) u[q] += (double)e[q];
}

// ---- single-CTA FP64 bottom solver (natural layout) -----------------------------------------
constexpr int kBottomThreads = 1024;

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

__device__ double bot_sum(double v, double* sm) {
    // deterministic tree reduction over the CTA
    const int t = threadIdx.x;
    sm[t] = v;
    __syncthreads();
    for (int o = kBottomThreads / 2; o > 0; o >>= 1) {
        if (t < o) sm[t] += sm[t + o];
        __syncthreads();
    }
    const double r = sm[0];
    __syncthreads();
    return r;
}

__device__ double bot_max(double v, double* sm) {
    const int t = threadIdx.x;
    sm[t] = v;
    __syncthreads();
    for (int o = kBottomThreads / 2; o > 0; o >>= 1) {
        if (t < o) sm[t] = fmax(sm[t], sm[t + o]);
        __syncthreads();
    }
    const double r = sm[0];
    __syncthreads();
    return r;
}

__device__ void bot_gsrb(const BotView& v, double* x, const double* f) {
    for (int colour = 0; colour < 2; ++colour) {
        for (int c = threadIdx.x; c < v.N; c += kBottomThreads) {
            const int i = c % v.n0, row = c / v.n0, j = row % v.n1, k = row / v.n1;
            if (((i + j + k) & 1) != colour) continue;
            x[c] = (f[c] + bot_arms(v, x, c)) * v.idg[c];
        }
        __syncthreads();
    }
}

__device__ void bot_apply(const BotView& v, const double* x, double* y) {
    for (int c = threadIdx.x; c < v.N; c += kBottomThreads) y[c] = v.dg[c] * x[c] - bot_arms(v, x, c);
    __syncthreads();
}

template <typename Tio>
__global__ void __launch_bounds__(kBottomThreads)
k_bottom(BotView v, Tio* __restrict__ xio, const Tio* __restrict__ fio, double* __restrict__ scr,
         int singular, int nub, double eps, int max_iter, int* __restrict__ iters) {
    __shared__ double sm[kBottomThreads];
    const int N = v.N;
    double* x = scr;
    double* f = scr + N;
    double* r = scr + 2 * N;
    double* rh = scr + 3 * N;
    double* p = scr + 4 * N;
    double* vv = scr + 5 * N;
    double* s = scr + 6 * N;
    double* t = scr + 7 * N;
    double* y = scr + 8 * N;
    const int tid = threadIdx.x;
    double loc = 0.0;
    for (int c = tid; c < N; c += kBottomThreads) {
        x[c] = (double)xio[c];
        f[c] = (double)fio[c];
        loc += f[c];
    }
    const double mean = bot_sum(loc, sm) / N;
    if (singular)
        for (int c = tid; c < N; c += kBottomThreads) f[c] -= mean;
    __syncthreads();
    for (int it = 0; it < nub; ++it) bot_gsrb(v, x, f);

    // r = f - A x
    bot_apply(v, x, t);
    loc = 0.0;
    for (int c = tid; c < N; c += kBottomThreads) {
        r[c] = f[c] - t[c];
        rh[c] = r[c];
        p[c] = 0.0;
        vv[c] = 0.0;
        loc = fmax(loc, fabs(r[c]));
    }
    const double r0 = bot_max(loc, sm);
    int count = 0;
    if (r0 > 0.0) {
        const double tol = eps * r0;
        double rho_old = 1.0, alpha = 1.0, omega = 1.0;
        for (int it = 0; it < max_iter; ++it) {
            ++count;
            loc = 0.0;
            for (int c = tid; c < N; c += kBottomThreads) loc += rh[c] * r[c];
            const double rho = bot_sum(loc, sm);
            if (rho == 0.0) break;
            const double beta = (rho / rho_old) * (alpha / omega);
            for (int c = tid; c < N; c += kBottomThreads) {
                p[c] = r[c] + beta * (p[c] - omega * vv[c]);
                y[c] = p[c] * v.idg[c];
            }
            __syncthreads();
            bot_apply(v, y, vv);
            loc = 0.0;
            for (int c = tid; c < N; c += kBottomThreads) loc += rh[c] * vv[c];
            const double rv = bot_sum(loc, sm);
            if (rv == 0.0) break;
            alpha = rho / rv;
            loc = 0.0;
            for (int c = tid; c < N; c += kBottomThreads) {
                s[c] = r[c] - alpha * vv[c];
                loc = fmax(loc, fabs(s[c]));
            }
            const double sn = bot_max(loc, sm);
            if (sn <= tol) {
                for (int c = tid; c < N; c += kBottomThreads) x[c] += alpha * y[c];
                __syncthreads();
                break;
            }
            // y now holds p/diag; keep it for the x update, use r as temporary for s/diag
            for (int c = tid; c < N; c += kBottomThreads) x[c] += alpha * y[c];
            for (int c = tid; c < N; c += kBottomThreads) y[c] = s[c] * v.idg[c];
            __syncthreads();
            bot_apply(v, y, t);
            double l1 = 0.0, l2 = 0.0;
            for (int c = tid; c < N; c += kBottomThreads) {
                l1 += t[c] * s[c];
                l2 += t[c] * t[c];
            }
            const double ts = bot_sum(l1, sm);
            const double tt = bot_sum(l2, sm);
            omega = tt > 0.0 ? ts / tt : 0.0;
            loc = 0.0;
            for (int c = tid; c < N; c += kBottomThreads) {
                x[c] += omega * y[c];
                r[c] = s[c] - omega * t[c];
                loc = fmax(loc, fabs(r[c]));
            }
            const double rn = bot_max(loc, sm);
            if (rn <= tol || omega == 0.0) break;
            rho_old = rho;
        }
    }
    for (int it = 0; it < nub; ++it) bot_gsrb(v, x, f);
    for (int c = tid; c < N; c += kBottomThreads) xio[c] = (Tio)x[c];
    if (tid == 0 && iters) atomicAdd(iters, count);
}

}  // namespace

// ---- launchers ------------------------------------------------------------------------------
template <typename T>
void launch_gsrb(const Dims& d, int colour, LevelArrays<T>& a, cudaStream_t s) {
    const int own = colour * d.half, oth = (colour ^ 1) * d.half;
    k_gsrb<T><<<ceil_div(d.half, kBlock), kBlock, 0, s>>>(
        d, colour, a.phi + own, a.phi + oth, a.f + own, a.bx + own, a.by + own, a.bz + own,
        a.bx + oth, a.by + oth, a.bz + oth, a.invdiag + own);
}

template <typename T>
void launch_resid_restrict(const Dims& fine, const Dims& coarse, const LevelArrays<T>& a, T* fc,
                           bool red_only, cudaStream_t s) {
    const int nb = ceil_div(coarse.ncell, kBlock);
    if (red_only)
        k_resid_restrict<T, true><<<nb, kBlock, 0, s>>>(fine, coarse, a.phi, a.f, a.bx, a.by, a.bz,
                                                        a.diag, fc);
    else
        k_resid_restrict<T, false><<<nb, kBlock, 0, s>>>(fine, coarse, a.phi, a.f, a.bx, a.by,
                                                         a.bz, a.diag, fc);
}

template <typename T>
void launch_prolong_add(const Dims& fine, const Dims& coarse, const BcDesc& bc, const T* ec,
                        T* phi_fine, cudaStream_t s) {
    k_prolong_add<T><<<ceil_div(fine.half, kBlock), kBlock, 0, s>>>(fine, coarse, bc, ec, phi_fine);
}

template <typename T>
void launch_resid_norm(const Dims& d, const LevelArrays<T>& a, bool red_only,
                       unsigned long long* maxbits, cudaStream_t s) {
    const int nb = ceil_div(d.half, kBlock);
    if (red_only)
        k_resid_norm<T, true><<<nb, kBlock, 0, s>>>(d, a.phi, a.f, a.bx, a.by, a.bz, a.diag, maxbits);
    else
        k_resid_norm<T, false><<<nb, kBlock, 0, s>>>(d, a.phi, a.f, a.bx, a.by, a.bz, a.diag,
                                                     maxbits);
}

void launch_resid64_to32(const Dims& d, const LevelArrays<double>& a, float* r32,
                         unsigned long long* maxbits, cudaStream_t s) {
    k_resid64_to32<<<ceil_div(d.half, kBlock), kBlock, 0, s>>>(d, a.phi, a.f, a.bx, a.by, a.bz,
                                                               a.diag, r32, maxbits);
}

void launch_accumulate(const Dims& d, double* phi, const float* e, cudaStream_t s) {
    k_accumulate<<<ceil_div(d.ncell, kBlock), kBlock, 0, s>>>(d.ncell, phi, e);
}

template <typename Tio>
void launch_bottom(const Dims& d, const LevelArrays<double>& a64, Tio* x, const Tio* f,
                   double* scratch, bool singular, int nub, double eps, int max_iter,
                   int* iter_counter, cudaStream_t s) {
    BotView v;
    v.n0 = d.n0;
    v.n1 = d.n1;
    v.n2 = d.n2;
    v.N = d.ncell;
    v.bx = a64.bx;
    v.by = a64.by;
    v.bz = a64.bz;
    v.dg = a64.diag;
    v.idg = a64.invdiag;
    k_bottom<Tio><<<1, kBottomThreads, 0, s>>>(v, x, f, scratch, singular ? 1 : 0, nub, eps,
                                               max_iter, iter_counter);
}

template void launch_gsrb<double>(const Dims&, int, LevelArrays<double>&, cudaStream_t);
template void launch_gsrb<float>(const Dims&, int, LevelArrays<float>&, cudaStream_t);
template void launch_resid_restrict<double>(const Dims&, const Dims&, const LevelArrays<double>&,
                                            double*, bool, cudaStream_t);
template void launch_resid_restrict<float>(const Dims&, const Dims&, const LevelArrays<float>&,
                                           float*, bool, cudaStream_t);
template void launch_prolong_add<double>(const Dims&, const Dims&, const BcDesc&, const double*,
                                         double*, cudaStream_t);
template void launch_prolong_add<float>(const Dims&, const Dims&, const BcDesc&, const float*,
                                        float*, cudaStream_t);
template void launch_resid_norm<double>(const Dims&, const LevelArrays<double>&, bool,
                                        unsigned long long*, cudaStream_t);
template void launch_resid_norm<float>(const Dims&, const LevelArrays<float>&, bool,
                                       unsigned long long*, cudaStream_t);
template void launch_bottom<double>(const Dims&, const LevelArrays<double>&, double*,
                                    const double*, double*, bool, int, double, int, int*,
                                    cudaStream_t);
template void launch_bottom<float>(const Dims&, const LevelArrays<double>&, float*, const float*,
                                   double*, bool, int, double, int, int*, cudaStream_t);

}  // namespace mac
