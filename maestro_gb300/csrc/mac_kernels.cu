// Multigrid kernels of the GB300 MAC projection: red/black Gauss-Seidel, defect + restriction,
// prolongation, residual norms and the single-CTA FP64 BiCGStab bottom solver.
//
// Arithmetic follows the FBoxLib cell-centred MG as described in MAESTRO's Docs/mg/mg.tex
// (:196-211 smoothers, :221-259 bottom solvers, :325-375 V-cycle flow); the level layout and
// the boundary trick are described in mac_internal.cuh.
#include <type_traits>

#include "mac_internal.cuh"
#include "mac_bottom.cuh"

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

__device__ __forceinline__ unsigned long long dbits(double v) {
    return (unsigned long long)__double_as_longlong(v);
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
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = tid & 31, wid = tid >> 5;
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = (lane < (int)((blockDim.x * blockDim.y) >> 5)) ? sm[lane] : 0ull;
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
            v = w > v ? w : v;
        }
    }
    return v;
}

// ---- red/black Gauss-Seidel half sweep (one colour) -----------------------------------------
template <typename T, bool SOR>
__global__ void __launch_bounds__(kBlock)
k_gsrb(Dims d, int colour, T* __restrict__ us, const T* __restrict__ uo, const T* __restrict__ fs,
       const T* __restrict__ bxs, const T* __restrict__ bys, const T* __restrict__ bzs,
       const T* __restrict__ bxo, const T* __restrict__ byo, const T* __restrict__ bzo,
       const T* __restrict__ ids, T omega) {
    pdl_wait();
    pdl_trigger();
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (h >= d.hn0 || j >= d.n1) return;
    const int q = (j + d.n1 * k) * d.hn0 + h;
    Nbr nb;
    split_nbrs(d, colour, h, j, k, nb);
    T acc = arms<T>(fs[q], q, nb, uo, bxs, bys, bzs, bxo, byo, bzo);
    if (SOR) {
        const T old = us[q];
        us[q] = fmaT(omega, acc * ids[q] - old, old);
    } else {
        us[q] = acc * ids[q];
    }
}

// Red/black half-sweep on a checkerboard-split FP32 level with 4 consecutive colour-half cells
// (h0 .. h0+3 of one row) per thread: every operand is a float4 load except the other colour's
// value (and x coefficient) one column outside the group.  Same per-cell arithmetic as k_gsrb.
// Requires hn0 % 4 == 0.
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float f4(const float4& v, int m) {
    return m == 0 ? v.x : m == 1 ? v.y : m == 2 ? v.z : v.w;
}

template <bool SOR>
__global__ void __launch_bounds__(kBlock)
k_gsrb4(Dims d, int colour, float* __restrict__ us, const float* __restrict__ uo,
        const float* __restrict__ fs, const float* __restrict__ bxs, const float* __restrict__ bys,
        const float* __restrict__ bzs, const float* __restrict__ bxo,
        const float* __restrict__ byo, const float* __restrict__ bzo,
        const float* __restrict__ ids, float omega) {
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    const int h0 = 4 * t;
    if (h0 >= d.hn0 || j >= d.n1) return;
    const int s = (colour + j + k) & 1;
    const int jm = (j == 0) ? d.n1 - 1 : j - 1;
    const int jp = (j == d.n1 - 1) ? 0 : j + 1;
    const int km = (k == 0) ? d.n2 - 1 : k - 1;
    const int kp = (k == d.n2 - 1) ? 0 : k + 1;
    const int row = (j + d.n1 * k) * d.hn0;
    const int q = row + h0;
    // column just outside the group on the side the parity needs (wrapped within the row)
    const int hx = s ? (h0 + 4 == d.hn0 ? 0 : h0 + 4) : (h0 == 0 ? d.hn0 - 1 : h0 - 1);
    const float4 f = ld4(fs + q), bx = ld4(bxs + q), by = ld4(bys + q), bz = ld4(bzs + q);
    const float4 id = ld4(ids + q);
    const float4 uc = ld4(uo + q);
    const float ux = uo[row + hx];
    const float4 bxn = ld4(bxo + q);
    const float bxx = bxo[row + hx];
    const float4 uym = ld4(uo + (jm + d.n1 * k) * d.hn0 + h0);
    const int qyp = (jp + d.n1 * k) * d.hn0 + h0;
    const float4 uyp = ld4(uo + qyp), byp = ld4(byo + qyp);
    const float4 uzm = ld4(uo + (j + d.n1 * km) * d.hn0 + h0);
    const int qzp = (j + d.n1 * kp) * d.hn0 + h0;
    const float4 uzp = ld4(uo + qzp), bzp = ld4(bzo + qzp);
    float out[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        // x-neighbours of cell i = 2 (h0 + m) + s: other-colour columns h-1+s (low), h+s (high)
        float ul, uh, bh;
        if (s) {
            ul = f4(uc, m);
            uh = m == 3 ? ux : f4(uc, m + 1);
            bh = m == 3 ? bxx : f4(bxn, m + 1);
        } else {
            ul = m == 0 ? ux : f4(uc, m - 1);
            uh = f4(uc, m);
            bh = f4(bxn, m);
        }
        float acc = f4(f, m);
        acc = fmaf(f4(bx, m), ul, acc);
        acc = fmaf(bh, uh, acc);
        acc = fmaf(f4(by, m), f4(uym, m), acc);
        acc = fmaf(f4(byp, m), f4(uyp, m), acc);
        acc = fmaf(f4(bz, m), f4(uzm, m), acc);
        acc = fmaf(f4(bzp, m), f4(uzp, m), acc);
        out[m] = acc * f4(id, m);
    }
    if (SOR) {
        const float4 o = ld4(us + q);
#pragma unroll
        for (int m = 0; m < 4; ++m) out[m] = fmaf(omega, out[m] - f4(o, m), f4(o, m));
    }
    *reinterpret_cast<float4*>(us + q) = make_float4(out[0], out[1], out[2], out[3]);
}

// ---- defect r = f - L u on the children of each coarse cell, averaged into the coarse rhs ---
template <typename T, bool RED_ONLY>
__global__ void __launch_bounds__(kBlock)
k_resid_restrict(Dims F, Dims C, const T* __restrict__ u, const T* __restrict__ f,
                 const T* __restrict__ bx, const T* __restrict__ by, const T* __restrict__ bz,
                 const T* __restrict__ dg, T* __restrict__ fc, T* __restrict__ ec) {
    pdl_wait();
    pdl_trigger();
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    if (I >= C.n0 || J >= C.n1) return;
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
    ec[ci] = T(0);   // the coarse correction starts from zero (no separate memset in the chain)
}

// ---- prolongation: u_fine += (bi/tri)linear interpolation of the coarse correction ----------
// Trilinear (bilinear in 2-D) cell-centred interpolation of the coarse correction, added to the
// 2^dm children of each coarse cell: one thread per coarse cell reads its 3x3x3 coarse
// neighbourhood (ghosts: periodic wrap, even/odd reflection for Neumann/Dirichlet, folded into
// the weights as signs) and interpolates separably, z then y then x, with weights 3/4 and 1/4.
template <typename T>
__device__ __forceinline__ void coarse_nb(int q, int n, int blo, int bhi, int& qm, int& qp, T& wm,
                                          T& wp) {
    wm = T(0.25);
    wp = T(0.25);
    if (q > 0) {
        qm = q - 1;
    } else if (blo == MAC_BC_PER) {
        qm = n - 1;
    } else {
        qm = 0;
        if (blo == MAC_BC_DIR) wm = T(-0.25);
    }
    if (q < n - 1) {
        qp = q + 1;
    } else if (bhi == MAC_BC_PER) {
        qp = 0;
    } else {
        qp = n - 1;
        if (bhi == MAC_BC_DIR) wp = T(-0.25);
    }
}

// BLACK_ONLY: add the correction to colour-1 cells only.  When post-smoothing follows, its first
// half-sweep overwrites every colour-0 cell without reading it (a red/black update reads only the
// other colour), so the colour-0 corrections would never be used: half the read-modify-write.
// uin: the fine values read (uin == u: in place; otherwise u gets uin + correction and the cells
// not updated keep u's values).
template <typename T, bool Z2, bool BLACK_ONLY>
__global__ void __launch_bounds__(kBlock)
k_prolong_add(Dims F, Dims C, BcDesc bc, const T* __restrict__ ec, T* u, const T* uin) {
    pdl_wait();
    pdl_trigger();
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    // every lane stays to the shuffles below; lanes outside the level compute nothing
    const bool valid = I < C.n0 && J < C.n1;
    int xs[3], ys[3], zs[3];
    T wxm, wxp, wym, wyp, wzm = T(0), wzp = T(0);
    xs[1] = I;
    ys[1] = J;
    zs[1] = K;
    coarse_nb<T>(I, C.n0, bc.lo[0], bc.hi[0], xs[0], xs[2], wxm, wxp);
    coarse_nb<T>(J, C.n1, bc.lo[1], bc.hi[1], ys[0], ys[2], wym, wyp);
    if (Z2) coarse_nb<T>(K, C.n2, bc.lo[2], bc.hi[2], zs[0], zs[2], wzm, wzp);
    auto cval = [&](int X, int Y, int Z) -> T {
        if (C.split) return ec[((X + Y + Z) & 1) * C.half + (Y + C.n1 * Z) * C.hn0 + (X >> 1)];
        return ec[X + C.n0 * (Y + C.n1 * Z)];
    };
    // Y[yc][zc]: the coarse column X interpolated in z, then y (9 coarse values)
    auto column = [&](int X, T (&Y)[2][2]) {
        T Zv[3][2];   // [y][zc]
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const int Yi = ys[b];
            const T c0 = cval(X, Yi, K);
            if (Z2) {
                const T t = T(0.75) * c0;
                Zv[b][0] = fmaT(wzm, cval(X, Yi, zs[0]), t);
                Zv[b][1] = fmaT(wzp, cval(X, Yi, zs[2]), t);
            } else {
                Zv[b][0] = c0;
                Zv[b][1] = c0;
            }
        }
#pragma unroll
        for (int zc = 0; zc < 2; ++zc) {
            const T t = T(0.75) * Zv[1][zc];
            Y[0][zc] = fmaT(wym, Zv[0][zc], t);
            Y[1][zc] = fmaT(wyp, Zv[2][zc], t);
        }
    };
    // Yv[a]: columns I-1, I, I+1.  The own column is computed here; the neighbouring ones come
    // from the lanes that computed them (same row, adjacent x) where those exist, else they are
    // computed again (warp edges, periodic wrap) or are the own column (walls).  The arithmetic
    // per column is the same whichever lane does it.
    // the fine values to update are loaded first: their DRAM latency overlaps the coarse loads
    // and the interpolation instead of following them
    const int hn0 = F.hn0, n1 = F.n1;
    constexpr int kNz = Z2 ? 2 : 1;
    T fold[kNz][2][2];
    if (valid) {
#pragma unroll
        for (int zc = 0; zc < kNz; ++zc)
#pragma unroll
            for (int yc = 0; yc < 2; ++yc) {
                const int base = (2 * J + yc + n1 * (Z2 ? 2 * K + zc : K)) * hn0 + I;
                const int c0 = (yc + zc) & 1;
                if (BLACK_ONLY) {
                    fold[zc][yc][0] = uin[F.half + base];
                } else {
                    fold[zc][yc][0] = uin[c0 * F.half + base];
                    fold[zc][yc][1] = uin[(c0 ^ 1) * F.half + base];
                }
            }
    }
    T Yv[3][2][2];
    if (valid) column(I, Yv[1]);
    else Yv[1][0][0] = Yv[1][0][1] = Yv[1][1][0] = Yv[1][1][1] = T(0);
    T lft[2][2], rgt[2][2];
#pragma unroll
    for (int yc = 0; yc < 2; ++yc)
#pragma unroll
        for (int zc = 0; zc < 2; ++zc) {
            lft[yc][zc] = __shfl_up_sync(0xffffffffu, Yv[1][yc][zc], 1);
            rgt[yc][zc] = __shfl_down_sync(0xffffffffu, Yv[1][yc][zc], 1);
        }
    if (!valid) return;
    const int lane = (threadIdx.x + blockDim.x * threadIdx.y) & 31;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const int a = side ? 2 : 0;
        const int X = xs[a];
        const bool from_lane = side ? (X == I + 1 && lane < 31 && threadIdx.x + 1 < blockDim.x)
                                    : (X == I - 1 && lane > 0 && threadIdx.x > 0);
        if (from_lane) {
#pragma unroll
            for (int yc = 0; yc < 2; ++yc)
#pragma unroll
                for (int zc = 0; zc < 2; ++zc) Yv[a][yc][zc] = side ? rgt[yc][zc] : lft[yc][zc];
        } else if (X == I) {
#pragma unroll
            for (int yc = 0; yc < 2; ++yc)
#pragma unroll
                for (int zc = 0; zc < 2; ++zc) Yv[a][yc][zc] = Yv[1][yc][zc];
        } else {
            column(X, Yv[a]);
        }
    }
#pragma unroll
    for (int zc = 0; zc < kNz; ++zc) {
#pragma unroll
        for (int yc = 0; yc < 2; ++yc) {
            const T t = T(0.75) * Yv[1][yc][zc];
            const int j = 2 * J + yc;
            const int k = Z2 ? 2 * K + zc : K;
            const int base = (j + n1 * k) * hn0 + I;
            const int c0 = (yc + zc) & 1;   // colour of child 2I (2I+2J+2K is even)
            if (BLACK_ONLY) {
                // the colour-1 child: 2I when c0 == 1, else 2I+1
                const T v = c0 ? fmaT(wxm, Yv[0][yc][zc], t) : fmaT(wxp, Yv[2][yc][zc], t);
                u[F.half + base] = fold[zc][yc][0] + v;
            } else {
                const T v0 = fmaT(wxm, Yv[0][yc][zc], t);
                const T v1 = fmaT(wxp, Yv[2][yc][zc], t);
                u[c0 * F.half + base] = fold[zc][yc][0] + v0;
                u[(c0 ^ 1) * F.half + base] = fold[zc][yc][1] + v1;
            }
        }
    }
}

// 3-D prolongation marching up z: a thread owns coarse column (I, J) for a chunk of planes and
// keeps the three coarse planes K-1, K, K+1 of its column's rows J-1, J, J+1 in registers (three
// loads a plane); the x-neighbour columns come from the adjacent lanes.  Each warp covers 30
// columns: lanes 0 and 31 only compute the columns left and right of them (periodic wrap or, at a
// wall, the edge column itself, which is what the wall reflection uses).  The arithmetic per
// fine cell is k_prolong_add's, operation for operation.
template <typename T, bool BLACK_ONLY>
__global__ void __launch_bounds__(kBlock)
k_prolong_z(Dims F, Dims C, BcDesc bc, const T* __restrict__ ec, T* __restrict__ u, int kc) {
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const int warp = (threadIdx.x >> 5) + (blockDim.x >> 5) * blockIdx.x;
    const int I = warp * 30 + lane - 1;
    const int J = blockIdx.y;
    const int K0 = blockIdx.z * kc;
    const int K1 = min(K0 + kc, C.n2);
    // the column this lane computes: its own, or the wrapped / clamped one beyond the ends
    const int X = I < 0 ? (bc.lo[0] == MAC_BC_PER ? C.n0 - 1 : 0)
                        : (I >= C.n0 ? (bc.hi[0] == MAC_BC_PER ? 0 : C.n0 - 1) : I);
    const bool out = lane >= 1 && lane <= 30 && I < C.n0;
    int ys[3];
    T wym, wyp, wxm = T(0), wxp = T(0);
    ys[1] = J;
    coarse_nb<T>(J, C.n1, bc.lo[1], bc.hi[1], ys[0], ys[2], wym, wyp);
    if (out) {
        int xm, xp;
        coarse_nb<T>(I, C.n0, bc.lo[0], bc.hi[0], xm, xp, wxm, wxp);
    }
    auto cval = [&](int Y, int Z) -> T {
        if (C.split) return ec[((X + Y + Z) & 1) * C.half + (Y + C.n1 * Z) * C.hn0 + (X >> 1)];
        return ec[X + C.n0 * (Y + C.n1 * Z)];
    };
    // planes K-1 (cm), K (c0), K+1 (cp) of rows ys[0..2], as coarse_nb indexes them (wrap or
    // clamp; the wall weight carries the sign)
    int zm, zp;
    T wzm, wzp;
    coarse_nb<T>(K0, C.n2, bc.lo[2], bc.hi[2], zm, zp, wzm, wzp);
    T cm[3], c0[3], cp[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        cm[b] = cval(ys[b], zm);
        c0[b] = cval(ys[b], K0);
        cp[b] = cval(ys[b], zp);
    }
    const int hn0 = F.hn0, n1 = F.n1;
#pragma unroll 2
    for (int K = K0; K < K1; ++K) {
        if (K > K0) {
            coarse_nb<T>(K, C.n2, bc.lo[2], bc.hi[2], zm, zp, wzm, wzp);
            // the window moves up one plane: K-1 <- K, K <- K+1, K+1 loaded (at a wall K-1 or
            // K+1 is plane K itself, which coarse_nb's index already says)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const T nk = cp[b];
                cm[b] = zm == K - 1 ? c0[b] : cval(ys[b], zm);
                c0[b] = nk;
                cp[b] = cval(ys[b], zp);
            }
        }
        T Zv[3][2];
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const T t = T(0.75) * c0[b];
            Zv[b][0] = fmaT(wzm, cm[b], t);
            Zv[b][1] = fmaT(wzp, cp[b], t);
        }
        T Yc[2][2], lft[2][2], rgt[2][2];
#pragma unroll
        for (int zc = 0; zc < 2; ++zc) {
            const T t = T(0.75) * Zv[1][zc];
            Yc[0][zc] = fmaT(wym, Zv[0][zc], t);
            Yc[1][zc] = fmaT(wyp, Zv[2][zc], t);
        }
#pragma unroll
        for (int yc = 0; yc < 2; ++yc)
#pragma unroll
            for (int zc = 0; zc < 2; ++zc) {
                lft[yc][zc] = __shfl_up_sync(0xffffffffu, Yc[yc][zc], 1);
                rgt[yc][zc] = __shfl_down_sync(0xffffffffu, Yc[yc][zc], 1);
            }
        if (!out) continue;
#pragma unroll
        for (int zc = 0; zc < 2; ++zc) {
#pragma unroll
            for (int yc = 0; yc < 2; ++yc) {
                const T t = T(0.75) * Yc[yc][zc];
                const int base = (2 * J + yc + n1 * (2 * K + zc)) * hn0 + I;
                const int cc = (yc + zc) & 1;   // colour of child 2I
                if (BLACK_ONLY) {
                    const T v = cc ? fmaT(wxm, lft[yc][zc], t) : fmaT(wxp, rgt[yc][zc], t);
                    u[F.half + base] += v;
                } else {
                    const T v0 = fmaT(wxm, lft[yc][zc], t);
                    const T v1 = fmaT(wxp, rgt[yc][zc], t);
                    u[cc * F.half + base] += v0;
                    u[(cc ^ 1) * F.half + base] += v1;
                }
            }
        }
    }
}

// ---- residual max-norm (FP64 accumulation of |r|) ---------------------------------------------
template <typename T, bool RED_ONLY>
__global__ void __launch_bounds__(kBlock)
k_resid_norm(Dims F, const T* __restrict__ u, const T* __restrict__ f, const T* __restrict__ bx,
             const T* __restrict__ by, const T* __restrict__ bz, const T* __restrict__ dg,
             unsigned long long* __restrict__ maxbits) {
    pdl_wait();
    pdl_trigger();
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    unsigned long long m = 0ull;
    if (h < F.hn0 && j < F.n1) {
        const int q = (j + F.n1 * k) * F.hn0 + h;
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
    if (threadIdx.x == 0 && threadIdx.y == 0 && m) atomicMax(maxbits, m);
}

// FP64 residual of the whole fine level, stored as FP32 (the refinement right-hand side).  Where
// phi is +0 on a cell and its six neighbours (the usual zero initial guess) the residual is f
// itself, except that -0 becomes +0 as (-0) + (+0) does in the FMA chain: that branch issues no
// FP64 instruction and reads no coefficient, with bitwise the chain's result.
__global__ void __launch_bounds__(kBlock)
k_resid64_to32(Dims F, const double* __restrict__ u, const double* __restrict__ f,
               const double* __restrict__ bx, const double* __restrict__ by,
               const double* __restrict__ bz, const double* __restrict__ dg,
               float* __restrict__ r32, unsigned long long* __restrict__ maxbits,
               float* __restrict__ e32) {
    pdl_wait();
    pdl_trigger();
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    unsigned long long m = 0ull;
    if (h < F.hn0 && j < F.n1) {
        const int q = (j + F.n1 * k) * F.hn0 + h;
#pragma unroll
        for (int colour = 0; colour < 2; ++colour) {
            const int off = colour * F.half, oth = (colour ^ 1) * F.half;
            Nbr nb;
            split_nbrs(F, colour, h, j, k, nb);
            const double* uo = u + oth;
            const double uc = u[off + q];
            const double v0 = uo[nb.xm], v1 = uo[nb.xp], v2 = uo[nb.ym], v3 = uo[nb.yp],
                         v4 = uo[nb.zm], v5 = uo[nb.zp];
            const unsigned long long any =
                dbits(uc) | dbits(v0) | dbits(v1) | dbits(v2) | dbits(v3) | dbits(v4) | dbits(v5);
            double r;
            if (any == 0ull) {
                const unsigned long long fb = dbits(f[off + q]);
                r = __longlong_as_double((long long)(fb == 0x8000000000000000ull ? 0ull : fb));
            } else {
                // the FMA order of arms(): x-, x+, y-, y+, z-, z+
                r = fma(-dg[off + q], uc, f[off + q]);
                r = fma(bx[off + q], v0, r);
                r = fma(bx[oth + nb.xp], v1, r);
                r = fma(by[off + q], v2, r);
                r = fma(by[oth + nb.yp], v3, r);
                r = fma(bz[off + q], v4, r);
                r = fma(bz[oth + nb.zp], v5, r);
            }
            r32[off + q] = to_float_rn(r);
            if (e32) e32[off + q] = 0.f;
            const unsigned long long b = abs_bits(r);
            m = b > m ? b : m;
        }
    }
    m = block_max_u64(m);
    if (threadIdx.x == 0 && threadIdx.y == 0 && m) atomicMax(maxbits, m);
}

// phi += e, four cells a thread (n % 4 == 0; the level-0 arrays always qualify), else one.  The
// FP32 -> FP64 widening takes the integer pipe (to_double), leaving the add the only FP64
// instruction of a cell.
template <int V>
__global__ void __launch_bounds__(kBlock)
k_accumulate(int n, double* __restrict__ u, const float* __restrict__ e) {
    pdl_wait();
    pdl_trigger();
    const int q = (blockIdx.x * blockDim.x + threadIdx.x) * V;
    if (q >= n) return;
    if (V == 4) {
        const float4 ev = *reinterpret_cast<const float4*>(e + q);
        double2 a = *reinterpret_cast<const double2*>(u + q);
        double2 b = *reinterpret_cast<const double2*>(u + q + 2);
        a.x += to_double(ev.x);
        a.y += to_double(ev.y);
        b.x += to_double(ev.z);
        b.y += to_double(ev.w);
        *reinterpret_cast<double2*>(u + q) = a;
        *reinterpret_cast<double2*>(u + q + 2) = b;
    } else {
        u[q] += to_double(e[q]);
    }
}

// Initial residual of a guess that is +0 everywhere: r = f (the FMA chain of k_resid64_to32
// gives f with -0 turned into +0), after f -= mean for a singular problem (the subtraction that
// would otherwise be its own pass).  Two cells a thread.
__global__ void __launch_bounds__(kBlock)
k_first_resid_zero(int n, double* __restrict__ f, const double* __restrict__ mean,
                   float* __restrict__ r32, float* __restrict__ e32,
                   unsigned long long* __restrict__ maxbits) {
    pdl_wait();
    pdl_trigger();
    const int q = (blockIdx.x * blockDim.x + threadIdx.x) * 2;
    unsigned long long m = 0ull;
    if (q < n) {
        double2 v = *reinterpret_cast<const double2*>(f + q);
        if (mean) {
            const double mu = *mean;
            v.x -= mu;
            v.y -= mu;
            *reinterpret_cast<double2*>(f + q) = v;
        }
        unsigned long long b0 = dbits(v.x), b1 = dbits(v.y);
        b0 = b0 == 0x8000000000000000ull ? 0ull : b0;
        b1 = b1 == 0x8000000000000000ull ? 0ull : b1;
        const double r0 = __longlong_as_double((long long)b0);
        const double r1 = __longlong_as_double((long long)b1);
        *reinterpret_cast<float2*>(r32 + q) = make_float2(to_float_rn(r0), to_float_rn(r1));
        *reinterpret_cast<float2*>(e32 + q) = make_float2(0.f, 0.f);
        const unsigned long long a0 = abs_bits(r0), a1 = abs_bits(r1);
        m = a0 > a1 ? a0 : a1;
    }
    m = block_max_u64(m);
    if (threadIdx.x == 0 && m) atomicMax(maxbits, m);
}

// ---- single-CTA FP64 bottom solver (natural layout): device code in mac_bottom.cuh -------------
constexpr int kBottomThreads = 1024;
constexpr int kBottomSmemCells = 1024;   // 7 + kBotScrPerCell doubles per cell: 204,800 B

// SMEM: the five operator arrays and the nine work vectors live in dynamic shared memory
// (levels of up to kBottomSmemCells cells, 128 threads), else in global scratch (1024 threads).
template <typename Tio, bool SMEM>
__global__ void __launch_bounds__(kBottomThreads)
k_bottom(BotView vin, Tio* __restrict__ xio, const Tio* __restrict__ fio, double* __restrict__ gscr,
         int singular, int nub, double eps, int max_iter, int* __restrict__ iters) {
    pdl_wait();
    pdl_trigger();
    __shared__ double sm[33];
    extern __shared__ double dsm[];
    const int N = vin.N;
    BotView v = vin;
    double* scr = gscr;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (SMEM) {
        double* ops = dsm;
        for (int c = tid; c < N; c += nt) {
            ops[c] = vin.bx[c];
            ops[N + c] = vin.by[c];
            ops[2 * N + c] = vin.bz[c];
            ops[3 * N + c] = vin.dg[c];
            ops[4 * N + c] = vin.idg[c];
        }
        v.bx = ops;
        v.by = ops + N;
        v.bz = ops + 2 * N;
        v.dg = ops + 3 * N;
        v.idg = ops + 4 * N;
        scr = dsm + 5 * N;
    }
    double* x = scr;
    double* f = scr + N;
    for (int c = tid; c < N; c += nt) {
        x[c] = (double)xio[c];
        f[c] = (double)fio[c];
    }
    __syncthreads();
    int count;
    if (SMEM)
        count = bottom_body<Sync128<false>>(v, x, f, scr + 2 * N, sm, singular, nub, eps, max_iter);
    else
        count = bottom_body<CtaSync>(v, x, f, scr + 2 * N, sm, singular, nub, eps, max_iter);
    __syncthreads();
    for (int c = tid; c < N; c += nt) xio[c] = (Tio)x[c];
    if (tid == 0 && iters) atomicAdd(iters, count);
}

}  // namespace

// ---- launchers ------------------------------------------------------------------------------
template <typename T>
void launch_gsrb(const Dims& d, int colour, LevelArrays<T>& a, cudaStream_t s, T omega) {
    const int own = colour * d.half, oth = (colour ^ 1) * d.half;
    const bool sor = omega != T(1);
    if constexpr (std::is_same<T, float>::value) {
        // four cells a thread pays off on large levels; small ones want more threads in flight
        if (d.hn0 % 4 == 0 && d.half >= (1 << 19)) {
            const Grid3 g4 = grid3(d.hn0 / 4, d.n1, d.n2);
            auto kern = sor ? k_gsrb4<true> : k_gsrb4<false>;
            launch_chain(kern, g4.grid, g4.block, 0, s, d, colour, a.phi + own,
                       (const float*)(a.phi + oth), (const float*)(a.f + own),
                       (const float*)(a.bx + own), (const float*)(a.by + own),
                       (const float*)(a.bz + own), (const float*)(a.bx + oth),
                       (const float*)(a.by + oth), (const float*)(a.bz + oth),
                       (const float*)(a.invdiag + own), omega);
            return;
        }
    }
    const Grid3 g = grid3(d.hn0, d.n1, d.n2);
    auto kern = sor ? k_gsrb<T, true> : k_gsrb<T, false>;
    launch_chain(kern, g.grid, g.block, 0, s, d, colour, a.phi + own, (const T*)(a.phi + oth),
               (const T*)(a.f + own), (const T*)(a.bx + own), (const T*)(a.by + own),
               (const T*)(a.bz + own), (const T*)(a.bx + oth), (const T*)(a.by + oth),
               (const T*)(a.bz + oth), (const T*)(a.invdiag + own), omega);
}

template <typename T>
void launch_resid_restrict(const Dims& fine, const Dims& coarse, const LevelArrays<T>& a, T* fc,
                           T* ec, bool red_only, cudaStream_t s) {
    const Grid3 g = grid3(coarse.n0, coarse.n1, coarse.n2);
    if (red_only)
        launch_chain(k_resid_restrict<T, true>, g.grid, g.block, 0, s, fine, coarse,
                   (const T*)a.phi, (const T*)a.f, (const T*)a.bx, (const T*)a.by, (const T*)a.bz,
                   (const T*)a.diag, fc, ec);
    else
        launch_chain(k_resid_restrict<T, false>, g.grid, g.block, 0, s, fine, coarse,
                   (const T*)a.phi, (const T*)a.f, (const T*)a.bx, (const T*)a.by, (const T*)a.bz,
                   (const T*)a.diag, fc, ec);
}

template <typename T>
void launch_prolong_add(const Dims& fine, const Dims& coarse, const BcDesc& bc, const T* ec,
                        T* phi_fine, bool black_only, cudaStream_t s, const T* phi_in) {
    const Grid3 g = grid3(coarse.n0, coarse.n1, coarse.n2);
    const T* uin = phi_in ? phi_in : phi_fine;
    if (std::is_same<T, double>::value && fine.rz == 2 && fine.split &&
        fine.ncell >= (1 << 22) && uin == phi_fine) {
        // z-marching kernel for large FP64 levels (measured: FP64 solve +2.4% at 256^3; the FP32
        // level-0 prolongation stays faster with one thread per coarse cell): warps of 30
        // columns, up to 8 warps a block along x; planes per thread as many as still leave ~48
        // warps per SM of GB300's 152 (the window's start costs three plane loads, a step one)
        const int warps = ceil_div(coarse.n0, 30);
        const int wpb = warps < 8 ? warps : 8;
        const long cols = (long)warps * coarse.n1;
        int kc = 16;
        while (kc > 2 && cols * ceil_div(coarse.n2, kc) < 152L * 48) kc >>= 1;
        const dim3 grid(ceil_div(warps, wpb), coarse.n1, ceil_div(coarse.n2, kc));
        if (black_only)
            launch_chain(k_prolong_z<T, true>, grid, dim3(32 * wpb), 0, s, fine, coarse, bc, ec,
                         phi_fine, kc);
        else
            launch_chain(k_prolong_z<T, false>, grid, dim3(32 * wpb), 0, s, fine, coarse, bc, ec,
                         phi_fine, kc);
    } else if (fine.rz == 2) {
        if (black_only)
            launch_chain(k_prolong_add<T, true, true>, g.grid, g.block, 0, s, fine, coarse, bc, ec,
                       phi_fine, uin);
        else
            launch_chain(k_prolong_add<T, true, false>, g.grid, g.block, 0, s, fine, coarse, bc, ec,
                       phi_fine, uin);
    } else {
        if (black_only)
            launch_chain(k_prolong_add<T, false, true>, g.grid, g.block, 0, s, fine, coarse, bc, ec,
                       phi_fine, uin);
        else
            launch_chain(k_prolong_add<T, false, false>, g.grid, g.block, 0, s, fine, coarse, bc, ec,
                       phi_fine, uin);
    }
}

template <typename T>
void launch_resid_norm(const Dims& d, const LevelArrays<T>& a, bool red_only,
                       unsigned long long* maxbits, cudaStream_t s) {
    const Grid3 g = grid3(d.hn0, d.n1, d.n2);
    if (red_only)
        launch_chain(k_resid_norm<T, true>, g.grid, g.block, 0, s, d, (const T*)a.phi,
                   (const T*)a.f, (const T*)a.bx, (const T*)a.by, (const T*)a.bz,
                   (const T*)a.diag, maxbits);
    else
        launch_chain(k_resid_norm<T, false>, g.grid, g.block, 0, s, d, (const T*)a.phi,
                   (const T*)a.f, (const T*)a.bx, (const T*)a.by, (const T*)a.bz,
                   (const T*)a.diag, maxbits);
}

void launch_resid64_to32(const Dims& d, const LevelArrays<double>& a, float* r32,
                         unsigned long long* maxbits, cudaStream_t s, float* e32) {
    const Grid3 g = grid3(d.hn0, d.n1, d.n2);
    launch_chain(k_resid64_to32, g.grid, g.block, 0, s, d, (const double*)a.phi,
               (const double*)a.f, (const double*)a.bx, (const double*)a.by, (const double*)a.bz,
               (const double*)a.diag, r32, maxbits, e32);
}

void launch_accumulate(const Dims& d, double* phi, const float* e, cudaStream_t s) {
    if (d.ncell % 4 == 0)
        launch_chain(k_accumulate<4>, dim3(ceil_div(d.ncell / 4, kBlock)), dim3(kBlock), 0, s,
                     d.ncell, phi, e);
    else
        launch_chain(k_accumulate<1>, dim3(ceil_div(d.ncell, kBlock)), dim3(kBlock), 0, s,
                     d.ncell, phi, e);
}

void launch_first_resid_zero(const Dims& d, double* f, const double* mean, float* r32,
                             float* e32, unsigned long long* maxbits, cudaStream_t s) {
    launch_chain(k_first_resid_zero, dim3(ceil_div(d.ncell / 2, kBlock)), dim3(kBlock), 0, s,
                 d.ncell, f, mean, r32, e32, maxbits);
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
    // small levels: 128 threads, operator and vectors in shared memory; large: one 1024-thread
    // CTA on global scratch
    const size_t smem = (size_t)(7 + kBotScrPerCell) * d.ncell * sizeof(double);
    if (d.ncell <= kBottomSmemCells)
        launch_chain(k_bottom<Tio, true>, dim3(1), dim3(128), smem, s, v, x, f, scratch,
                   singular ? 1 : 0, nub, eps, max_iter, iter_counter);
    else
        launch_chain(k_bottom<Tio, false>, dim3(1), dim3(kBottomThreads), 0, s, v, x, f, scratch,
                   singular ? 1 : 0, nub, eps, max_iter, iter_counter);
}

// Opt the shared-memory bottom solver into more than 48 KB of dynamic shared memory (called once
// per context, outside any stream capture).
int prepare_kernels() {
    const int bytes = (7 + kBotScrPerCell) * kBottomSmemCells * (int)sizeof(double);
    if (cudaFuncSetAttribute(k_bottom<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess ||
        cudaFuncSetAttribute(k_bottom<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) {
        cudaGetLastError();
        return MAC_ERR_CUDA;
    }
    return MAC_OK;
}

template void launch_gsrb<double>(const Dims&, int, LevelArrays<double>&, cudaStream_t, double);
template void launch_gsrb<float>(const Dims&, int, LevelArrays<float>&, cudaStream_t, float);
template void launch_resid_restrict<double>(const Dims&, const Dims&, const LevelArrays<double>&,
                                            double*, double*, bool, cudaStream_t);
template void launch_resid_restrict<float>(const Dims&, const Dims&, const LevelArrays<float>&,
                                            float*, float*, bool, cudaStream_t);
template void launch_prolong_add<double>(const Dims&, const Dims&, const BcDesc&, const double*,
                                         double*, bool, cudaStream_t, const double*);
template void launch_prolong_add<float>(const Dims&, const Dims&, const BcDesc&, const float*,
                                         float*, bool, cudaStream_t, const float*);
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
