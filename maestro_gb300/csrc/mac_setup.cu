// Fine-level setup and finishing kernels of the GB300 MAC projection: face coefficients,
// coarse-level coefficients, right-hand side, velocity correction, layout conversion and the
// gather / scatter between the caller's per-box fabs and the whole-domain device arrays.
//
// Reference steps (Source/macproject.f90):
//   154-158  mult_edge_by_1d_coeff(umac, ...,.true.)   -> fused into k_rhs and k_correct
//   175-179  divumac, rh = -(div(beta0 U) - macrhs)     -> k_rhs        (385-398, 457-480)
//   182-193  mk_mac_coeffs + beta0 multiply             -> k_fine_coef  (698-738, 577-609)
//   229      mkumac                                     -> k_correct    (908-975)
//   232-236  divide out beta0                           -> fused into k_correct
//   245-251  multifab_fill_boundary                     -> k_scatter_faces (ghost faces)
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <vector>

#include "mac_internal.cuh"

namespace mac {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ int lidx(const Dims& d, int i, int j, int k) { return level_index(d, i, j, k); }

struct FineParams {
    int n[3];
    int bc_lo[3], bc_hi[3];
    int va;          // vertical direction
    int p;           // beta0 exponent (1 or 2); 0 = no beta0
    int active[3];
    double ih2[3];
};


// Per-layer factor tables (see kTab* in mac_internal.cuh), one thread per vertical index r.
// beta0 on the low face of a cell in layer r: beta0[r] for the horizontal directions,
// beta0_edge[r] for the vertical one (mult_edge_by_1d_coeff, Source/macproject.f90:577-609).
__global__ void k_beta0_tables(int nr, int va, int p, const double* __restrict__ b0,
                               const double* __restrict__ b0e, double3 h, double* __restrict__ tab,
                               float* __restrict__ fac32, int vper, int vdlo, int vdhi) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r > nr) return;
    const double hh[3] = {h.x, h.y, h.z};
    const int st = nr + 1;
    const double bc = p ? b0[r < nr ? r : nr - 1] : 1.0;
    const double be = p ? b0e[r] : 1.0;
    for (int d = 0; d < 3; ++d) {
        const double b = d == va ? be : bc;
        const double bp = p == 2 ? b * b : (p == 1 ? b : 1.0);
        tab[(kTabFac0 + d) * st + r] = bp * 2.0 / (hh[d] * hh[d]);
        tab[(kTabG0 + d) * st + r] = b / hh[d];
        tab[(kTabK0 + d) * st + r] = hh[d] / b;
    }
    // FP32 tables of the on-the-fly finest-level kernels (OtfParams)
    const double hv = hh[va];
    const double bcp = p == 2 ? bc * bc : (p == 1 ? bc : 1.0);
    fac32[0 * st + r] = (float)(bcp * 2.0 / (hh[0] * hh[0]));
    fac32[1 * st + r] = (float)(bcp * 2.0 / (hh[1] * hh[1]));
    if (r < nr) {
        const double bl = p ? b0e[r] : 1.0, bh = p ? b0e[r + 1] : 1.0;
        const double fl = (p == 2 ? bl * bl : (p == 1 ? bl : 1.0)) * 2.0 / (hv * hv);
        const double fh = (p == 2 ? bh * bh : (p == 1 ? bh : 1.0)) * 2.0 / (hv * hv);
        const bool wl = r == 0 && !vper, wh = r == nr - 1 && !vper;
        fac32[2 * st + r] = wl ? 0.f : (float)fl;
        fac32[3 * st + r] = wh ? 0.f : (float)fh;
        // Dirichlet wall: 2 beta'_wall = 2 fac/(2 rho) = fac / rho, here the fac part
        fac32[4 * st + r] = (float)((wl && vdlo ? fl : 0.0) + (wh && vdhi ? fh : 0.0));
    } else {
        fac32[2 * st + r] = 0.f;
        fac32[3 * st + r] = 0.f;
        fac32[4 * st + r] = 0.f;
    }
}

// beta' on the low faces of every fine cell, Dirichlet wall planes, density check.
// beta'_d = fac_d[layer] / (rho_a + rho_b)  (= beta0^p 2/(rho_a + rho_b) / h_d^2)
__device__ __forceinline__ void fine_face(const FineParams& P, int dd, int cd, int nd, int q,
                                          int stride, double rc, const double* __restrict__ rho,
                                          double fac, double fhi, double* out, int li,
                                          double* wl, double* wh, int plane) {
    double v = 0.0;
    const bool per = P.bc_lo[dd] == MAC_BC_PER;
    if (cd > 0)
        v = fac * recip_nr(rc + rho[q - stride]);
    else if (per)
        v = fac * recip_nr(rc + rho[q + (nd - 1) * stride]);
    out[li] = v;
    if (cd == 0 && P.bc_lo[dd] == MAC_BC_DIR) wl[plane] = fac * recip_nr(rc + rc);
    if (cd == nd - 1 && P.bc_hi[dd] == MAC_BC_DIR) wh[plane] = fhi * recip_nr(rc + rc);
}

__global__ void __launch_bounds__(kBlock)
k_fine_coef(FineParams P, Dims d, const double* __restrict__ rho, const double* __restrict__ tab,
            double* __restrict__ bx, double* __restrict__ by, double* __restrict__ bz,
            double* __restrict__ wlo0, double* __restrict__ whi0, double* __restrict__ wlo1,
            double* __restrict__ whi1, double* __restrict__ wlo2, double* __restrict__ whi2,
            int* __restrict__ err, float* __restrict__ rho32) {
    const int n0 = P.n[0], n1 = P.n[1], n2 = P.n[2];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n0 || j >= n1) return;
    const int q = i + n0 * (j + n1 * k);
    const double rc = rho[q];
    if (!positive_finite(rc)) atomicOr(err, 1);
    const int li = lidx(d, i, j, k);
    if (rho32) rho32[li] = to_float_rn(rc);
    const bool v2 = P.va == 2;
    const int r = v2 ? k : j;                       // vertical index (3-D: z, 2-D: y)
    const int st = (v2 ? n2 : n1) + 1;
    const double* f0 = tab + kTabFac0 * st;
    const double* f1 = tab + (kTabFac0 + 1) * st;
    const double* f2 = tab + (kTabFac0 + 2) * st;
    // x: horizontal
    fine_face(P, 0, i, n0, q, 1, rc, rho, f0[r], f0[r], bx, li, wlo0, whi0, j + n1 * k);
    // y: horizontal in 3-D, vertical in 2-D
    fine_face(P, 1, j, n1, q, n0, rc, rho, f1[r], v2 ? f1[r] : f1[r + 1], by, li, wlo1, whi1,
              i + n0 * k);
    // z: vertical in 3-D, absent in 2-D
    if (P.active[2])
        fine_face(P, 2, k, n2, q, n0 * n1, rc, rho, f2[r], f2[r + 1], bz, li, wlo2, whi2,
                  i + n0 * j);
    else
        bz[li] = 0.0;
}

struct DiagParams {
    int bc_lo[3], bc_hi[3];
    int any_dir;
    const double* wl[3];
    const double* wh[3];
};

// diag = alpha + sum of the six face coefficients (+ 2 beta'_wall on Dirichlet faces); optional
// 1/diag in FP64 and FP32 copies of diag and 1/diag (mixed precision).
__global__ void __launch_bounds__(kBlock)
k_build_diag(Dims d, DiagParams P, const double* __restrict__ bx, const double* __restrict__ by,
             const double* __restrict__ bz, const double* __restrict__ alpha,
             double* __restrict__ dg, double* __restrict__ idg, float* __restrict__ dg32,
             float* __restrict__ idg32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= d.n0 || j >= d.n1) return;
    const int me = lidx(d, i, j, k);
    const int ip = i == d.n0 - 1 ? 0 : i + 1;
    const int jp = j == d.n1 - 1 ? 0 : j + 1;
    const int kp = k == d.n2 - 1 ? 0 : k + 1;
    double s = alpha ? alpha[me] : 0.0;
    s += bx[me] + bx[lidx(d, ip, j, k)];
    s += by[me] + by[lidx(d, i, jp, k)];
    s += bz[me] + bz[lidx(d, i, j, kp)];
    if (P.any_dir) {
        if (i == 0 && P.bc_lo[0] == MAC_BC_DIR) s += 2.0 * P.wl[0][j + d.n1 * k];
        if (i == d.n0 - 1 && P.bc_hi[0] == MAC_BC_DIR) s += 2.0 * P.wh[0][j + d.n1 * k];
        if (j == 0 && P.bc_lo[1] == MAC_BC_DIR) s += 2.0 * P.wl[1][i + d.n0 * k];
        if (j == d.n1 - 1 && P.bc_hi[1] == MAC_BC_DIR) s += 2.0 * P.wh[1][i + d.n0 * k];
        if (k == 0 && P.bc_lo[2] == MAC_BC_DIR) s += 2.0 * P.wl[2][i + d.n0 * j];
        if (k == d.n2 - 1 && P.bc_hi[2] == MAC_BC_DIR) s += 2.0 * P.wh[2][i + d.n0 * j];
    }
    dg[me] = s;
    if (idg) idg[me] = recip_nr(s);
    if (dg32) {
        const float sf = (float)s;
        dg32[me] = sf;
        idg32[me] = 1.0f / sf;
    }
}

// Coarse low-face coefficients: mean of the fine low faces tiling the coarse face, / 4 for h^2.
__global__ void __launch_bounds__(kBlock)
k_coarsen_coef(Dims F, Dims C, const double* __restrict__ fbx, const double* __restrict__ fby,
               const double* __restrict__ fbz, const double* __restrict__ falpha,
               double* __restrict__ cbx, double* __restrict__ cby, double* __restrict__ cbz,
               double* __restrict__ calpha, float* __restrict__ cbx32, float* __restrict__ cby32,
               float* __restrict__ cbz32) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    if (I >= C.n0 || J >= C.n1) return;
    const int rz = F.rz;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int b = 0; b < rz; ++b)
        for (int a = 0; a < 2; ++a) {
            sx += fbx[lidx(F, 2 * I, 2 * J + a, rz * K + b)];
            sy += fby[lidx(F, 2 * I + a, 2 * J, rz * K + b)];
        }
    if (rz == 2)
        for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) sz += fbz[lidx(F, 2 * I + a, 2 * J + b, 2 * K)];
    const int me = lidx(C, I, J, K);
    const double w = rz == 2 ? 0.0625 : 0.125;   // 1/4 (h^2) times the mean over 2*rz faces
    const double vx = w * sx, vy = w * sy, vz = rz == 2 ? 0.0625 * sz : 0.0;
    cbx[me] = vx;
    cby[me] = vy;
    cbz[me] = vz;
    if (cbx32) {
        cbx32[me] = (float)vx;
        cby32[me] = (float)vy;
        cbz32[me] = (float)vz;
    }
    if (falpha) {
        double sa = 0.0;
        for (int b = 0; b < rz; ++b)
            for (int a1 = 0; a1 < 2; ++a1)
                for (int a0 = 0; a0 < 2; ++a0) sa += falpha[lidx(F, 2 * I + a0, 2 * J + a1, rz * K + b)];
        calpha[me] = sa * (rz == 2 ? 0.125 : 0.25);
    }
}

// Coarse Dirichlet wall plane: mean of the fine wall faces, / 4 for h^2.
__global__ void k_coarsen_wall(int np0, int np1, int r0, int r1, int fp0,
                               const double* __restrict__ fw, double* __restrict__ cw) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np0 * np1) return;
    const int P0 = q % np0, P1 = q / np0;
    double s = 0.0;
    for (int b = 0; b < r1; ++b)
        for (int a = 0; a < r0; ++a) s += fw[(r0 * P0 + a) + fp0 * (r1 * P1 + b)];
    cw[q] = 0.25 * s * (r0 * r1 == 4 ? 0.25 : (r0 * r1 == 2 ? 0.5 : 1.0));
}

__global__ void k_to_f32(int n, const double* __restrict__ a, float* __restrict__ b) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) b[q] = (float)a[q];
}

struct RhsParams {
    int n[3];
    int dm, va, have_beta0;
    double idx[3];   // 1/dx
};

// f = -(div(beta0 U) - macrhs) (FROM_RH: f = rh, already a natural cell array) in the level-0
// layout, with per-block partials: FP64 sum (fixed order) and max/min of f as ordered bit
// patterns (integer pipe).  U is scaled by beta0 face by face as mult_edge_by_1d_coeff does (x/y
// faces by beta0(k), the vertical faces by beta0_edge(k)) before the differences.  Each block
// covers a (bx x by) tile of rows over kRhsPlanes planes so the partials stay few.
template <int DM, bool FROM_RH>
__global__ void __launch_bounds__(kBlock)
k_rhs(RhsParams P, Dims d, const double* __restrict__ ux, const double* __restrict__ uy,
      const double* __restrict__ uz, const double* __restrict__ macrhs,
      const double* __restrict__ tab, double* __restrict__ f, double* __restrict__ partial,
      const double* __restrict__ phi_nat, double* __restrict__ phi_l0) {
    __shared__ double ssum[8];
    __shared__ unsigned long long smax[8], smin[8], sor[8];
    const int n0 = P.n[0], n1 = P.n[1], n2 = P.n[2];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k0 = blockIdx.z * kRhsPlanes;
    double sum = 0.0;
    unsigned long long mx = 0ull, mn = ~0ull;
    // OR of the guess's bit patterns: 0 when phi is +0 everywhere (no guess given: unknown)
    unsigned long long por = phi_nat ? 0ull : ~0ull;
    if (i < n0 && j < n1) {
        const int st = P.n[DM - 1] + 1;
        for (int k = k0; k < k0 + kRhsPlanes && k < n2; ++k) {
            const int q = i + n0 * (j + n1 * k);
            double v;
            if (FROM_RH) {
                v = macrhs[q];
            } else {
                const int r = DM == 3 ? k : j;
                const int fx = i + (n0 + 1) * (j + n1 * k);
                const int fy = i + n0 * (j + (n1 + 1) * k);
                // div(beta0 U) with beta0/dx folded into per-layer factors
                double dv = (ux[fx + 1] - ux[fx]) * tab[kTabG0 * st + r];
                if (DM == 3) {
                    dv = fma(uy[fy + n0] - uy[fy], tab[(kTabG0 + 1) * st + r], dv);
                    const double* g = tab + (kTabG0 + 2) * st;
                    dv = fma(uz[q + n0 * n1], g[r + 1], dv);
                    dv = fma(-uz[q], g[r], dv);
                } else {
                    const double* g = tab + (kTabG0 + 1) * st;
                    dv = fma(uy[fy + n0], g[r + 1], dv);
                    dv = fma(-uy[fy], g[r], dv);
                }
                v = macrhs ? macrhs[q] - dv : -dv;
            }
            const int li = lidx(d, i, j, k);
            f[li] = v;
            // the initial guess moves to the level-0 layout in the same pass (this kernel is
            // bound by the FP64 pipe, the copy rides along in its memory slack)
            if (phi_nat) {
                const double g = phi_nat[q];
                phi_l0[li] = g;
                por |= (unsigned long long)__double_as_longlong(g);
            }
            sum += v;
            const unsigned long long o = ordered_bits(v);
            mx = o > mx ? o : mx;
            mn = o < mn ? o : mn;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        const unsigned long long a = __shfl_down_sync(0xffffffffu, mx, o);
        const unsigned long long b = __shfl_down_sync(0xffffffffu, mn, o);
        mx = a > mx ? a : mx;
        mn = b < mn ? b : mn;
        por |= __shfl_down_sync(0xffffffffu, por, o);
    }
    const int t = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = t & 31, wid = t >> 5, nw = (blockDim.x * blockDim.y) >> 5;
    if (lane == 0) {
        ssum[wid] = sum;
        smax[wid] = mx;
        smin[wid] = mn;
        sor[wid] = por;
    }
    __syncthreads();
    if (t == 0) {
        double s = 0.0;
        unsigned long long a = 0ull, b = ~0ull, o = 0ull;
        for (int w = 0; w < nw; ++w) {
            s += ssum[w];
            a = smax[w] > a ? smax[w] : a;
            b = smin[w] < b ? smin[w] : b;
            o |= sor[w];
        }
        const int blk = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        partial[kRhsPartials * blk + 0] = s;
        partial[kRhsPartials * blk + 1] = __longlong_as_double((long long)a);
        partial[kRhsPartials * blk + 2] = __longlong_as_double((long long)b);
        partial[kRhsPartials * blk + 3] = __longlong_as_double((long long)o);
    }
}

// Deterministic final reduction of the k_rhs partials: mean (singular problems) and
// ||f - mean||_inf; NaN if anything is not finite; [5] the OR of the guess's bit patterns.
__global__ void k_rhs_final(int nblocks, int ncell, int singular, const double* __restrict__ partial,
                            double* __restrict__ scalars) {
    __shared__ double ssum[32];
    __shared__ unsigned long long smax[32], smin[32], sor[32];
    double s = 0.0;
    unsigned long long mx = 0ull, mn = ~0ull, por = 0ull;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        const double* pb = partial + kRhsPartials * b;
        s += pb[0];
        const unsigned long long a = (unsigned long long)__double_as_longlong(pb[1]);
        const unsigned long long c = (unsigned long long)__double_as_longlong(pb[2]);
        mx = a > mx ? a : mx;
        mn = c < mn ? c : mn;
        por |= (unsigned long long)__double_as_longlong(pb[3]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        const unsigned long long a = __shfl_down_sync(0xffffffffu, mx, o);
        const unsigned long long c = __shfl_down_sync(0xffffffffu, mn, o);
        mx = a > mx ? a : mx;
        mn = c < mn ? c : mn;
        por |= __shfl_down_sync(0xffffffffu, por, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        ssum[wid] = s;
        smax[wid] = mx;
        smin[wid] = mn;
        sor[wid] = por;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        unsigned long long a = 0ull, c = ~0ull, o = 0ull;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            t += ssum[w];
            a = smax[w] > a ? smax[w] : a;
            c = smin[w] < c ? smin[w] : c;
            o |= sor[w];
        }
        scalars[5] = __longlong_as_double((long long)o);
        const double vmax = from_ordered_bits(a), vmin = from_ordered_bits(c);
        const double mean = singular ? t / ncell : 0.0;
        scalars[0] = mean;
        scalars[1] = fmax(vmax - mean, mean - vmin);
        if (!isfinite(t) || !isfinite(vmax) || !isfinite(vmin)) scalars[1] = NAN;
        scalars[2] = t;
        scalars[3] = vmax;
        scalars[4] = vmin;
    }
}

__global__ void k_sub_mean(int n, double* __restrict__ f, const double* __restrict__ scalars) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) f[q] -= scalars[0];
}

struct CorrParams {
    int n[3];
    int dir, va, have_beta0;
    int bc_lo, bc_hi;
    double idx;  // 1/dx
    double h2;   // h_dir^2 (beta = beta' * h2)
};

// U = (beta0 U - beta_f G phi) / beta0 = U - beta' (h / beta0) (phi_hi - phi_lo) on every face
// normal to P.dir (natural face layout); beta' = beta_f / h^2 is the stored coefficient, h/beta0 a
// per-layer factor.  Neumann walls keep U; Dirichlet walls use the ghost -phi_boundary.
__global__ void __launch_bounds__(kBlock)
k_correct(CorrParams P, Dims d, double* __restrict__ u, const double* __restrict__ phi,
          const double* __restrict__ bd, const double* __restrict__ wlo,
          const double* __restrict__ whi, const double* __restrict__ tab,
          double* __restrict__ phi_nat) {
    const int dir = P.dir;
    const int m0 = P.n[0] + (dir == 0), m1 = P.n[1] + (dir == 1);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= m0 || j >= m1) return;
    const int q = i + m0 * (j + m1 * k);
    const int qd = dir == 0 ? i : (dir == 1 ? j : k);
    const int nd = dir == 0 ? P.n[0] : (dir == 1 ? P.n[1] : P.n[2]);
    const bool v2 = P.va == 2;
    const int r = v2 ? k : j;
    const int st = (v2 ? P.n[2] : P.n[1]) + 1;
    const double kap = tab[(kTabK0 + dir) * st + r];
    const int plane = dir == 0 ? (j + P.n[1] * k) : dir == 1 ? (i + P.n[0] * k) : (i + P.n[0] * j);
    // cells on the low (a) and high (b) side of the face, periodic wrap at the boundary faces
    const int di = dir == 0, dj = dir == 1, dk = dir == 2;
    double beta = 0.0, dphi = 0.0;
    if (qd > 0 && qd < nd) {
        const int chi = lidx(d, i, j, k);
        beta = bd[chi];
        dphi = phi[chi] - phi[lidx(d, i - di, j - dj, k - dk)];
    } else if ((qd == 0 && P.bc_lo == MAC_BC_PER) || (qd == nd && P.bc_hi == MAC_BC_PER)) {
        const int chi = lidx(d, di ? 0 : i, dj ? 0 : j, dk ? 0 : k);
        beta = bd[chi];
        dphi = phi[chi] - phi[lidx(d, di ? nd - 1 : i, dj ? nd - 1 : j, dk ? nd - 1 : k)];
    } else if (qd == 0) {
        if (P.bc_lo == MAC_BC_DIR) {
            beta = wlo[plane];
            dphi = 2.0 * phi[lidx(d, i, j, k)];
        }
    } else if (P.bc_hi == MAC_BC_DIR) {
        beta = whi[plane];
        dphi = -2.0 * phi[lidx(d, i - di, j - dj, k - dk)];
    }
    // beta == 0 (a wall face without Dirichlet) leaves the face alone; tested on the bit pattern
    // so that no FP64 comparison occupies the FP64 pipe
    if ((unsigned long long)__double_as_longlong(beta) << 1) u[q] = fma(-(beta * kap), dphi, u[q]);
    // the x-direction pass also returns phi to the natural layout (one cell per x face but the
    // last; this kernel is bound by the FP64 pipe, the copy rides along)
    if (phi_nat && i < P.n[0]) phi_nat[i + P.n[0] * (j + P.n[1] * k)] = phi[lidx(d, i, j, k)];
}

template <typename T>
__global__ void k_nat_to_l0(Dims d, const T* __restrict__ src, T* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= d.n0 || j >= d.n1) return;
    dst[lidx(d, i, j, k)] = src[i + d.n0 * (j + d.n1 * k)];
}

template <typename T>
__global__ void k_l0_to_nat(Dims d, const T* __restrict__ src, T* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= d.n0 || j >= d.n1) return;
    dst[i + d.n0 * (j + d.n1 * k)] = src[lidx(d, i, j, k)];
}

// ---- caller box layout <-> whole-domain natural arrays --------------------------------------
struct GatherParams {
    int n[3];       // domain cells (internal 3-D)
    int dm;
    int dir;        // -1: cell field; 0..2: faces normal to dir
    int bc_per[3];  // periodic flag per direction
};

// Whole-domain array <- valid region of every box.  Faces: each box writes lo..hi along dir,
// and hi+1 only at the domain's high end.  One warp per x-row of a box (rows = (j, k) pairs),
// lanes striding x with four loads in flight, so that fabs read over the host link (page-locked
// host memory) keep enough requests outstanding.  Block (32, kRowsPerBlock), grid (row blocks,
// boxes).
constexpr int kRowsPerBlock = 8;

__global__ void __launch_bounds__(32 * kRowsPerBlock)
k_gather(GatherParams P, const BoxDesc* __restrict__ boxes, double* __restrict__ dst) {
    const BoxDesc& B = boxes[blockIdx.y];
    const int e0 = B.hi[0] - B.lo[0] + 1 + (P.dir == 0);
    const int e1 = B.hi[1] - B.lo[1] + 1 + (P.dir == 1);
    const int e2 = B.hi[2] - B.lo[2] + 1 + (P.dir == 2);
    const int row = blockIdx.x * kRowsPerBlock + threadIdx.y;
    if (row >= e1 * e2) return;
    const int b = row % e1, c = row / e1;
    const int gj = B.lo[1] + b, gk = B.lo[2] + c;
    if (P.dir == 1 && b == e1 - 1 && gj != P.n[1]) return;   // the next box's low face
    if (P.dir == 2 && c == e2 - 1 && gk != P.n[2]) return;
    const int ev = (P.dir == 0 && B.hi[0] + 1 != P.n[0]) ? e0 - 1 : e0;
    const int m0 = P.n[0] + (P.dir == 0), m1 = P.n[1] + (P.dir == 1);
    const int g0 = B.ng, g1 = B.ng, g2 = P.dm == 3 ? B.ng : 0;
    const double* s =
        B.ptr + B.comp_off + g0 + (long)B.ext[0] * ((b + g1) + (long)B.ext[1] * (c + g2));
    double* d = dst + B.lo[0] + (long)m0 * (gj + (long)m1 * gk);
    for (int a0 = threadIdx.x; a0 < ev; a0 += 128) {
        double v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = a0 + 32 * q < ev ? s[a0 + 32 * q] : 0.0;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (a0 + 32 * q < ev) d[a0 + 32 * q] = v[q];
    }
}

// Every entry of every fab (valid + ghosts) <- whole-domain array, periodic wrap; ghosts outside
// a non-periodic domain boundary are left untouched.  One warp per fab row, as k_gather.
__global__ void __launch_bounds__(32 * kRowsPerBlock)
k_scatter(GatherParams P, const BoxDesc* __restrict__ boxes, const double* __restrict__ src) {
    const BoxDesc& B = boxes[blockIdx.y];
    const int row = blockIdx.x * kRowsPerBlock + threadIdx.y;
    if (row >= B.ext[1] * B.ext[2]) return;
    const int b = row % B.ext[1], c = row / B.ext[1];
    const int g[3] = {B.ng, B.ng, P.dm == 3 ? B.ng : 0};
    int gc[3] = {0, B.lo[1] - g[1] + b, B.lo[2] - g[2] + c};
    for (int dd = 1; dd < 3; ++dd) {
        const int lim = P.n[dd] + (P.dir == dd ? 1 : 0);
        if (gc[dd] < 0 || gc[dd] >= lim) {
            if (!P.bc_per[dd]) return;
            gc[dd] = (gc[dd] % P.n[dd] + P.n[dd]) % P.n[dd];
        }
    }
    const int m0 = P.n[0] + (P.dir == 0), m1 = P.n[1] + (P.dir == 1);
    const int lim0 = m0, x0 = B.lo[0] - g[0];
    const double* s = src + (long)m0 * (gc[1] + (long)m1 * gc[2]);
    double* d = const_cast<double*>(B.ptr) + (long)B.ext[0] * (b + (long)B.ext[1] * c);
    const int e0 = B.ext[0];
    for (int a0 = threadIdx.x; a0 < e0; a0 += 128) {
        double v[4];
        bool ok[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int a = a0 + 32 * q;
            int gi = x0 + a;
            ok[q] = a < e0;
            if (gi < 0 || gi >= lim0) {
                if (P.bc_per[0])
                    gi = (gi % P.n[0] + P.n[0]) % P.n[0];
                else
                    ok[q] = false;
            }
            v[q] = ok[q] ? s[gi] : 0.0;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (ok[q]) d[a0 + 32 * q] = v[q];
    }
}

// Launch grid of k_gather / k_scatter: enough row blocks for the largest box.
dim3 box_rows_grid(const mac_ctx* c, int dir, int ng, bool with_ghosts) {
    long rows = 1;
    for (int b = 0; b < c->g.nboxes; ++b) {
        long r = 1;
        for (int d = 1; d < 3; ++d) {
            const int g = (d < c->dm && with_ghosts) ? ng : 0;
            const int lo = d < c->dm ? c->box_lo[3 * b + d] : 0;
            const int hi = d < c->dm ? c->box_hi[3 * b + d] : 0;
            r *= (long)(hi - lo + 1 + (dir == d ? 1 : 0) + 2 * g);
        }
        rows = r > rows ? r : rows;
    }
    return dim3((unsigned)ceil_div((int)rows, kRowsPerBlock), (unsigned)c->g.nboxes);
}

// beta' from caller-supplied face coefficients (natural face layout), Dirichlet wall planes,
// and the optional Helmholtz alpha moved into the level-0 layout.
__global__ void __launch_bounds__(kBlock)
k_fine_coef_faces(FineParams P, Dims d, const double* __restrict__ fx,
                  const double* __restrict__ fy, const double* __restrict__ fz,
                  const double* __restrict__ alpha_nat, double* __restrict__ alpha_l0,
                  double* __restrict__ bx, double* __restrict__ by, double* __restrict__ bz,
                  double* __restrict__ wlo0, double* __restrict__ whi0, double* __restrict__ wlo1,
                  double* __restrict__ whi1, double* __restrict__ wlo2, double* __restrict__ whi2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= P.n[0] || j >= P.n[1]) return;
    const int q = i + P.n[0] * (j + P.n[1] * k);
    const int c[3] = {i, j, k};
    const int li = lidx(d, i, j, k);
    const double* fin[3] = {fx, fy, fz};
    double* out[3] = {bx, by, bz};
    double* wl[3] = {wlo0, wlo1, wlo2};
    double* wh[3] = {whi0, whi1, whi2};
    if (alpha_l0) alpha_l0[li] = alpha_nat[q];
#pragma unroll
    for (int dd = 0; dd < 3; ++dd) {
        if (!P.active[dd]) {
            out[dd][li] = 0.0;
            continue;
        }
        const int m0 = P.n[0] + (dd == 0), m1 = P.n[1] + (dd == 1);
        const int flo = i + m0 * (j + m1 * k);
        const int stride = dd == 0 ? 1 : dd == 1 ? m0 : m0 * m1;
        const double blo = fin[dd][flo];
        out[dd][li] = (c[dd] > 0 || P.bc_lo[dd] == MAC_BC_PER) ? blo * P.ih2[dd] : 0.0;
        const int plane = dd == 0 ? (j + P.n[1] * k) : dd == 1 ? (i + P.n[0] * k) : (i + P.n[0] * j);
        if (c[dd] == 0 && P.bc_lo[dd] == MAC_BC_DIR) wl[dd][plane] = blo * P.ih2[dd];
        if (c[dd] == P.n[dd] - 1 && P.bc_hi[dd] == MAC_BC_DIR)
            wh[dd][plane] = fin[dd][flo + stride] * P.ih2[dd];
    }
}

Dims level0_dims(const mac_ctx* c) { return c->lev[0].d; }

}  // namespace

// ------------------------------------------------------------------------------------------
namespace {

DiagParams diag_params(const mac_ctx* c, const Level& L) {
    DiagParams D;
    D.any_dir = 0;
    for (int d = 0; d < 3; ++d) {
        D.bc_lo[d] = c->bc_lo[d];
        D.bc_hi[d] = c->bc_hi[d];
        D.wl[d] = L.wall[d][0];
        D.wh[d] = L.wall[d][1];
        D.any_dir |= (c->bc_lo[d] == MAC_BC_DIR || c->bc_hi[d] == MAC_BC_DIR) ? 1 : 0;
    }
    return D;
}

bool mixed(const mac_ctx* c) { return c->o.precision == MAC_PREC_MIXED; }

// diag (+ 1/diag in FP64 where an FP64 smoother or the bottom solve reads it, + FP32 copies
// for the mixed-precision inner cycle) of level l.  A mixed-precision context still runs FP64
// V-cycles of level 0 when an AMR hierarchy is set (the coarse correction of the composite
// cycle), so every level then needs the FP64 1/diag too.
int build_diag(mac_ctx* c, int l, bool fp32) {
    Level& L = c->lev[l];
    const bool need_inv64 = !mixed(c) || l == c->nlevels - 1 || c->amr != nullptr;
    const Grid3 g = grid3(L.d.n0, L.d.n1, L.d.n2);
    k_build_diag<<<g.grid, g.block, 0, c->stream>>>(
        L.d, diag_params(c, L), L.a64.bx, L.a64.by, L.a64.bz, L.alpha, L.a64.diag,
        need_inv64 ? L.a64.invdiag : nullptr, fp32 ? L.a32.diag : nullptr,
        fp32 ? L.a32.invdiag : nullptr);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    return MAC_OK;
}

}  // namespace

int setup_fine_coefficients(mac_ctx* c, const double* beta0, const double* beta0e) {
    Level& L = c->lev[0];
    FineParams P;
    for (int d = 0; d < 3; ++d) {
        P.n[d] = c->n[d];
        P.bc_lo[d] = c->bc_lo[d];
        P.bc_hi[d] = c->bc_hi[d];
        P.active[d] = d < c->dm ? 1 : 0;
        P.ih2[d] = 1.0 / (L.h[d] * L.h[d]);
    }
    P.va = c->va;
    P.p = beta0 ? (c->o.use_alt_energy_fix ? 2 : 1) : 0;
    MAC_CUDA_TRY(cudaMemsetAsync(c->red.counters, 0, 4 * sizeof(int), c->stream));
    const int nr = c->n[c->va];
    k_beta0_tables<<<ceil_div(nr + 1, 128), 128, 0, c->stream>>>(
        nr, c->va, P.p, beta0, beta0e, make_double3(L.h[0], L.h[1], L.h[2]), c->b0tab, c->fac32,
        c->bc_lo[c->va] == MAC_BC_PER ? 1 : 0, c->bc_lo[c->va] == MAC_BC_DIR ? 1 : 0,
        c->bc_hi[c->va] == MAC_BC_DIR ? 1 : 0);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    const Grid3 g = grid3(L.d.n0, L.d.n1, L.d.n2);
    k_fine_coef<<<g.grid, g.block, 0, c->stream>>>(
        P, L.d, c->rho, c->b0tab, L.a64.bx, L.a64.by, L.a64.bz, L.wall[0][0], L.wall[0][1],
        L.wall[1][0], L.wall[1][1], L.wall[2][0], L.wall[2][1], c->red.counters + 1,
        c->otf ? c->rho32 : nullptr);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    return build_diag(c, 0, mixed(c) && !c->otf);
}

int setup_coarse_levels(mac_ctx* c) {
    const bool fp32 = mixed(c);
    for (int l = 1; l < c->nlevels; ++l) {
        Level& F = c->lev[l - 1];
        Level& C = c->lev[l];
        const Grid3 g = grid3(C.d.n0, C.d.n1, C.d.n2);
        k_coarsen_coef<<<g.grid, g.block, 0, c->stream>>>(
            F.d, C.d, F.a64.bx, F.a64.by, F.a64.bz, F.alpha, C.a64.bx, C.a64.by, C.a64.bz, C.alpha,
            fp32 ? C.a32.bx : nullptr, fp32 ? C.a32.by : nullptr, fp32 ? C.a32.bz : nullptr);
        MAC_CUDA_TRY(cudaGetLastError());
        ++c->issued;
        for (int d = 0; d < 3; ++d)
            for (int s = 0; s < 2; ++s) {
                if (!C.wall[d][s]) continue;
                // plane directions: the two directions other than d, x fastest
                const int p0 = d == 0 ? 1 : 0, p1 = d == 2 ? 1 : 2;
                const int r[3] = {2, 2, F.d.rz};
                const int cn[3] = {C.d.n0, C.d.n1, C.d.n2};
                const int fn[3] = {F.d.n0, F.d.n1, F.d.n2};
                const int np0 = cn[p0], np1 = cn[p1];
                k_coarsen_wall<<<ceil_div((long)np0 * np1, kBlock), kBlock, 0, c->stream>>>(
                    np0, np1, r[p0], r[p1], fn[p0], F.wall[d][s], C.wall[d][s]);
                MAC_CUDA_TRY(cudaGetLastError());
                ++c->issued;
            }
        int rc = build_diag(c, l, fp32);
        if (rc) return rc;
    }
    return issue_bottom_inverse(c);
}

// FP32 copies of the finest level's operator for the mixed-precision inner cycle when its
// coefficients are not computed on the fly (mac_multigrid: face coefficients given).
int setup_fp32_copies(mac_ctx* c) {
    if (c->otf) return MAC_OK;
    Level& L = c->lev[0];
    const int n = L.d.ncell;
    const double* src[3] = {L.a64.bx, L.a64.by, L.a64.bz};
    float* dst[3] = {L.a32.bx, L.a32.by, L.a32.bz};
    for (int a = 0; a < 3; ++a) {
        k_to_f32<<<ceil_div(n, kBlock), kBlock, 0, c->stream>>>(n, src[a], dst[a]);
        MAC_CUDA_TRY(cudaGetLastError());
        ++c->issued;
    }
    return MAC_OK;
}

namespace {

int launch_rhs(mac_ctx* c, const double* macrhs, bool from_rh, const double* phi_nat) {
    Level& L = c->lev[0];
    RhsParams P;
    for (int d = 0; d < 3; ++d) {
        P.n[d] = c->n[d];
        P.idx[d] = 1.0 / c->dx[d];
    }
    P.dm = c->dm;
    P.va = c->va;
    P.have_beta0 = 1;
    const Grid3 g = rhs_grid(c->n);
    const int nb = (int)(g.grid.x * g.grid.y * g.grid.z);
    if (nb > c->red.nblocks_partial) return MAC_ERR_INVALID;   // buffer sized by rhs_grid
    if (c->dm == 3) {
        if (from_rh)
            k_rhs<3, true><<<g.grid, g.block, 0, c->stream>>>(P, L.d, nullptr, nullptr, nullptr, macrhs,
                                                              c->b0tab, L.a64.f, c->red.partial, phi_nat, L.a64.phi);
        else
            k_rhs<3, false><<<g.grid, g.block, 0, c->stream>>>(P, L.d, c->u[0], c->u[1], c->u[2], macrhs,
                                                               c->b0tab, L.a64.f, c->red.partial, phi_nat, L.a64.phi);
    } else {
        if (from_rh)
            k_rhs<2, true><<<g.grid, g.block, 0, c->stream>>>(P, L.d, nullptr, nullptr, nullptr, macrhs,
                                                              c->b0tab, L.a64.f, c->red.partial, phi_nat, L.a64.phi);
        else
            k_rhs<2, false><<<g.grid, g.block, 0, c->stream>>>(P, L.d, c->u[0], c->u[1], nullptr, macrhs,
                                                               c->b0tab, L.a64.f, c->red.partial, phi_nat, L.a64.phi);
    }
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    k_rhs_final<<<1, 1024, 0, c->stream>>>(nb, L.d.ncell, c->singular ? 1 : 0, c->red.partial,
                                           c->red.scalars);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    // the mean of a singular problem comes off f in the solve's first pass over f (run_solve)
    c->mean_pending = c->singular;
    return MAC_OK;
}

}  // namespace

void launch_sub_mean(mac_ctx* c) {
    Level& L = c->lev[0];
    k_sub_mean<<<ceil_div(L.d.ncell, kBlock), kBlock, 0, c->stream>>>(L.d.ncell, L.a64.f,
                                                                     c->red.scalars);
}

int setup_rhs(mac_ctx* c, const double* macrhs, bool have_beta0, const double* phi_nat) {
    (void)have_beta0;   // the factor tables hold beta0 = 1 when there is none
    return launch_rhs(c, macrhs, false, phi_nat);
}

int correct_velocity(mac_ctx* c, bool have_beta0, const std::function<int(int)>* after_dir,
                     double* phi_nat_out) {
    Level& L = c->lev[0];
    const double* bd[3] = {L.a64.bx, L.a64.by, L.a64.bz};
    for (int d = 0; d < c->dm; ++d) {
        CorrParams P;
        for (int e = 0; e < 3; ++e) P.n[e] = c->n[e];
        P.dir = d;
        P.va = c->va;
        P.have_beta0 = have_beta0 ? 1 : 0;
        P.bc_lo = c->bc_lo[d];
        P.bc_hi = c->bc_hi[d];
        P.idx = 1.0 / c->dx[d];
        P.h2 = c->dx[d] * c->dx[d];
        const Grid3 g = grid3(c->n[0] + (d == 0), c->n[1] + (d == 1), c->n[2] + (d == 2));
        k_correct<<<g.grid, g.block, 0, c->stream>>>(P, L.d, c->u[d], L.a64.phi, bd[d],
                                                     L.wall[d][0], L.wall[d][1], c->b0tab,
                                                     d == 0 ? phi_nat_out : nullptr);
        MAC_CUDA_TRY(cudaGetLastError());
        ++c->issued;
        if (after_dir) {
            int rc = (*after_dir)(d);
            if (rc) return rc;
        }
    }
    return MAC_OK;
}

namespace {
template <typename T>
int nat_to_l0(mac_ctx* c, const T* src, T* dst) {
    const Dims d = level0_dims(c);
    const Grid3 g = grid3(d.n0, d.n1, d.n2);
    k_nat_to_l0<T><<<g.grid, g.block, 0, c->stream>>>(d, src, dst);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    return MAC_OK;
}
template <typename T>
int l0_to_nat(mac_ctx* c, const T* src, T* dst) {
    const Dims d = level0_dims(c);
    const Grid3 g = grid3(d.n0, d.n1, d.n2);
    k_l0_to_nat<T><<<g.grid, g.block, 0, c->stream>>>(d, src, dst);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    return MAC_OK;
}
}  // namespace

int natural_to_level0(mac_ctx* c, const double* src, double* dst) { return nat_to_l0(c, src, dst); }
int level0_to_natural(mac_ctx* c, const double* src, double* dst) { return l0_to_nat(c, src, dst); }
int natural_to_level0(mac_ctx* c, const float* src, float* dst) { return nat_to_l0(c, src, dst); }
int level0_to_natural(mac_ctx* c, const float* src, float* dst) { return l0_to_nat(c, src, dst); }

// ---- box tables ----------------------------------------------------------------------------
namespace {

constexpr int kBoxSlots = 16;

constexpr int kBoxChunk = 64;   // 64 descriptors fit the 4 KB kernel-parameter space
struct BoxChunk {
    int n;
    BoxDesc b[kBoxChunk];
};
__global__ void k_put_boxes(BoxChunk ch, BoxDesc* __restrict__ dst) {
    for (int q = threadIdx.x; q < ch.n; q += blockDim.x) dst[q] = ch.b[q];
}

struct SlotCursor {
    int next = 0;
};
thread_local SlotCursor g_slot;

// Fill one slot of the pinned box table and push it to the device; returns the device table.
int fill_boxes(mac_ctx* c, int dir, int ng, int ncomp, int comp, const double* const* ptrs,
               int ptr_kind, bool to_device_staging, BoxDesc** dev_table, size_t* total_elems,
               std::vector<size_t>* offsets) {
    const int nb = c->g.nboxes;
    const int slot = g_slot.next;
    g_slot.next = (g_slot.next + 1) % kBoxSlots;
    BoxDesc* h = c->h_boxes + (size_t)slot * nb;
    size_t off = 0;
    offsets->assign(nb, 0);
    for (int b = 0; b < nb; ++b) {
        BoxDesc& B = h[b];
        for (int d = 0; d < 3; ++d) {
            B.lo[d] = d < c->dm ? c->box_lo[3 * b + d] - c->g.domain_lo[d] : 0;
            B.hi[d] = d < c->dm ? c->box_hi[3 * b + d] - c->g.domain_lo[d] : 0;
            const int g = d < c->dm ? ng : 0;
            B.ext[d] = B.hi[d] - B.lo[d] + 1 + (dir == d ? 1 : 0) + 2 * g;
        }
        B.ng = ng;
        const size_t comp_elems = (size_t)B.ext[0] * B.ext[1] * B.ext[2];
        B.comp_off = 0;
        if (ptr_kind == MAC_PTR_DEVICE) {
            B.ptr = ptrs[b] + comp_elems * comp;
        } else {
            B.ptr = c->staging + off;
            (*offsets)[b] = off;
            off += comp_elems;
        }
        (void)ncomp;
        (void)to_device_staging;
    }
    *total_elems = off;
    BoxDesc* d = c->d_boxes + (size_t)slot * nb;
    // uploaded as kernel parameters, not by a copy: a host -> device copy on the main stream would
    // queue on the copy engine behind the transfer stream's bulk input copies
    for (int b0 = 0; b0 < nb; b0 += kBoxChunk) {
        BoxChunk ch;
        ch.n = std::min(kBoxChunk, nb - b0);
        for (int q = 0; q < ch.n; ++q) ch.b[q] = h[b0 + q];
        k_put_boxes<<<1, 32, 0, c->stream>>>(ch, d + b0);
        MAC_CUDA_TRY(cudaGetLastError());
    }
    *dev_table = d;
    return MAC_OK;
}

int ensure_staging(mac_ctx* c, size_t elems) {
    if (elems <= c->staging_elems) return MAC_OK;
    if (c->staging) {
        MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
        if (c->xfer) MAC_CUDA_TRY(cudaStreamSynchronize(c->xfer));
        cudaFree(c->staging);
        c->staging = nullptr;
    }
    cudaError_t e = cudaMalloc(&c->staging, elems * sizeof(double));
    if (e != cudaSuccess) {
        c->staging_elems = 0;
        return MAC_ERR_ALLOC;
    }
    c->staging_elems = elems;
    return MAC_OK;
}

GatherParams gparams(const mac_ctx* c, int dir) {
    GatherParams P;
    for (int d = 0; d < 3; ++d) {
        P.n[d] = c->n[d];
        P.bc_per[d] = (d < c->dm && c->bc_lo[d] == MAC_BC_PER) ? 1 : 0;
    }
    P.dm = c->dm;
    P.dir = dir;
    return P;
}

// Elements of one box's fab (one component) in element offset order of the fab list.
size_t fab_elems(const mac_ctx* c, int b, int dir, int ng) {
    size_t e = 1;
    for (int d = 0; d < 3; ++d) {
        const int g = d < c->dm ? ng : 0;
        const int lo = d < c->dm ? c->box_lo[3 * b + d] : 0;
        const int hi = d < c->dm ? c->box_hi[3 * b + d] : 0;
        e *= (size_t)(hi - lo + 1 + (dir == d ? 1 : 0) + 2 * g);
    }
    return e;
}

cudaEvent_t next_event(mac_ctx* c) {
    cudaEvent_t e = c->xev[c->xev_next];
    c->xev_next = (c->xev_next + 1) % (int)(sizeof(c->xev) / sizeof(c->xev[0]));
    return e;
}

double* staging_take(mac_ctx* c, size_t elems) {
    if (c->staging_cursor + elems > c->staging_elems) return nullptr;
    double* p = c->staging + c->staging_cursor;
    c->staging_cursor += elems;
    return p;
}

// Region of a fab that k_scatter writes, per direction as [lo, hi] in fab-local indices: every
// entry whose global index lies in the domain, or in a periodic direction.
void written_region(const mac_ctx* c, int b, int dir, int ng, int lo[3], int hi[3], int ext[3]) {
    for (int d = 0; d < 3; ++d) {
        if (d >= c->dm) {
            lo[d] = hi[d] = 0;
            ext[d] = 1;
            continue;
        }
        const int blo = c->box_lo[3 * b + d] - c->g.domain_lo[d];
        const int bhi = c->box_hi[3 * b + d] - c->g.domain_lo[d];
        ext[d] = bhi - blo + 1 + (dir == d ? 1 : 0) + 2 * ng;
        const bool per = c->bc_lo[d] == MAC_BC_PER;
        const int lim = c->n[d] + (dir == d ? 1 : 0);
        const int g0 = blo - ng;   // global index of fab entry 0
        lo[d] = per ? 0 : std::max(0, -g0);
        hi[d] = per ? ext[d] - 1 : std::min(ext[d] - 1, lim - 1 - g0);
    }
}

}  // namespace

size_t host_fab_elems(const mac_ctx* c, int dir, int ng) {
    size_t tot = 0;
    for (int b = 0; b < c->g.nboxes; ++b) tot += fab_elems(c, b, dir, ng);
    return tot;
}

// Make room for the staging regions of one host-pointer call and start carving at offset 0.
int staging_reserve(mac_ctx* c, size_t total_elems) {
    int rc = ensure_staging(c, total_elems);
    if (rc) return rc;
    c->staging_cursor = 0;
    return MAC_OK;
}

int gather_begin(mac_ctx* c, int ptr_kind, const double* const* fabs, int ng, int ncomp, int comp,
                 int dir, double* dst, PendingGather* pg) {
    pg->ptr_kind = ptr_kind;
    pg->fabs = fabs;
    pg->ng = ng;
    pg->ncomp = ncomp;
    pg->comp = comp;
    pg->dir = dir;
    pg->dst = dst;
    pg->region = nullptr;
    pg->ev = nullptr;
    if (ptr_kind != MAC_PTR_HOST) return MAC_OK;
    const size_t need = host_fab_elems(c, dir, ng);
    if (c->staging_cursor + need > c->staging_elems) {
        // a call that did not reserve (or an unplanned array): grow after the pending work
        MAC_CUDA_TRY(cudaStreamSynchronize(c->xfer));
        MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
        int rc = ensure_staging(c, need);
        if (rc) return rc;
        c->staging_cursor = 0;
    }
    pg->region = staging_take(c, need);
    size_t off = 0;
    for (int b = 0; b < c->g.nboxes; ++b) {
        const size_t e = fab_elems(c, b, dir, ng);
        MAC_CUDA_TRY(cudaMemcpyAsync(pg->region + off, fabs[b] + e * comp, e * sizeof(double),
                                     cudaMemcpyHostToDevice, c->xfer));
        off += e;
    }
    pg->ev = next_event(c);
    MAC_CUDA_TRY(cudaEventRecord(pg->ev, c->xfer));
    return MAC_OK;
}

int gather_end(mac_ctx* c, const PendingGather& pg) {
    BoxDesc* table = nullptr;
    size_t tot = 0;
    std::vector<size_t> offs;
    int rc;
    if (pg.ptr_kind == MAC_PTR_HOST) {
        MAC_CUDA_TRY(cudaStreamWaitEvent(c->stream, pg.ev, 0));
        // the staged copy holds one component per fab, contiguous in box order
        std::vector<const double*> ptrs(c->g.nboxes);
        size_t off = 0;
        for (int b = 0; b < c->g.nboxes; ++b) {
            ptrs[b] = pg.region + off;
            off += fab_elems(c, b, pg.dir, pg.ng);
        }
        rc = fill_boxes(c, pg.dir, pg.ng, 1, 0, ptrs.data(), MAC_PTR_DEVICE, false, &table, &tot,
                        &offs);
    } else {
        rc = fill_boxes(c, pg.dir, pg.ng, pg.ncomp, pg.comp, pg.fabs, MAC_PTR_DEVICE, false, &table,
                        &tot, &offs);
    }
    if (rc) return rc;
    const GatherParams P = gparams(c, pg.dir);
    k_gather<<<box_rows_grid(c, pg.dir, pg.ng, false), dim3(32, kRowsPerBlock), 0, c->stream>>>(
        P, table, pg.dst);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    return MAC_OK;
}

namespace {

int gather_common(mac_ctx* c, int ptr_kind, const double* const* fabs, int ng, int ncomp, int comp,
                  int dir, double* dst) {
    PendingGather pg;
    int rc = gather_begin(c, ptr_kind, fabs, ng, ncomp, comp, dir, dst, &pg);
    return rc ? rc : gather_end(c, pg);
}

// Whole-domain array -> every fab.  Host pointers: the kernel fills a staging copy of the fabs on
// the main stream and the copy engines bring back, per fab, only the region the kernel wrote, so
// the host entries it leaves alone (ghosts outside non-periodic walls) keep their values.  The
// copies complete on the transfer stream; the caller synchronises it before returning.
int scatter_common(mac_ctx* c, int ptr_kind, double* const* fabs, int ng, int dir,
                   const double* src) {
    BoxDesc* table = nullptr;
    size_t tot = 0;
    std::vector<size_t> offs;
    double* region = nullptr;
    std::vector<const double*> ptrs(c->g.nboxes);
    if (ptr_kind == MAC_PTR_HOST) {
        const size_t need = host_fab_elems(c, dir, ng);
        if (c->staging_cursor + need > c->staging_elems) {
            MAC_CUDA_TRY(cudaStreamSynchronize(c->xfer));
            MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
            int rc = ensure_staging(c, need);
            if (rc) return rc;
            c->staging_cursor = 0;
        }
        region = staging_take(c, need);
        size_t off = 0;
        for (int b = 0; b < c->g.nboxes; ++b) {
            ptrs[b] = region + off;
            off += fab_elems(c, b, dir, ng);
        }
    } else {
        for (int b = 0; b < c->g.nboxes; ++b) ptrs[b] = fabs[b];
    }
    int rc = fill_boxes(c, dir, ng, 1, 0, ptrs.data(), MAC_PTR_DEVICE, false, &table, &tot, &offs);
    if (rc) return rc;
    const GatherParams P = gparams(c, dir);
    k_scatter<<<box_rows_grid(c, dir, ng, true), dim3(32, kRowsPerBlock), 0, c->stream>>>(P, table,
                                                                                           src);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    if (ptr_kind != MAC_PTR_HOST) return MAC_OK;
    cudaEvent_t ev = next_event(c);
    MAC_CUDA_TRY(cudaEventRecord(ev, c->stream));
    MAC_CUDA_TRY(cudaStreamWaitEvent(c->xfer, ev, 0));
    for (int b = 0; b < c->g.nboxes; ++b) {
        int lo[3], hi[3], ext[3];
        written_region(c, b, dir, ng, lo, hi, ext);
        double* sdev = const_cast<double*>(ptrs[b]);
        if (lo[0] == 0 && hi[0] == ext[0] - 1 && lo[1] == 0 && hi[1] == ext[1] - 1) {
            // whole rows and planes: one linear copy of planes lo[2] .. hi[2]
            const size_t plane = (size_t)ext[0] * ext[1];
            MAC_CUDA_TRY(cudaMemcpyAsync(fabs[b] + plane * lo[2], sdev + plane * lo[2],
                                         plane * (hi[2] - lo[2] + 1) * sizeof(double),
                                         cudaMemcpyDeviceToHost, c->xfer));
        } else {
            cudaMemcpy3DParms p = {};
            p.srcPtr = make_cudaPitchedPtr(sdev, ext[0] * sizeof(double), ext[0], ext[1]);
            p.dstPtr = make_cudaPitchedPtr(fabs[b], ext[0] * sizeof(double), ext[0], ext[1]);
            p.srcPos = make_cudaPos(lo[0] * sizeof(double), lo[1], lo[2]);
            p.dstPos = p.srcPos;
            p.extent = make_cudaExtent((hi[0] - lo[0] + 1) * sizeof(double), hi[1] - lo[1] + 1,
                                       hi[2] - lo[2] + 1);
            p.kind = cudaMemcpyDeviceToHost;
            MAC_CUDA_TRY(cudaMemcpy3DAsync(&p, c->xfer));
        }
    }
    return MAC_OK;
}

}  // namespace

int gather_cells(mac_ctx* c, int ptr_kind, const double* const* fabs, int ng, int ncomp, int comp,
                 double* dst) {
    return gather_common(c, ptr_kind, fabs, ng, ncomp, comp, -1, dst);
}
int gather_faces(mac_ctx* c, int ptr_kind, const double* const* fabs, int ng, int dir,
                 double* dst) {
    return gather_common(c, ptr_kind, fabs, ng, 1, 0, dir, dst);
}
int scatter_cells(mac_ctx* c, int ptr_kind, double* const* fabs, int ng, const double* src) {
    return scatter_common(c, ptr_kind, fabs, ng, -1, src);
}
int scatter_faces(mac_ctx* c, int ptr_kind, double* const* fabs, int ng, int dir,
                  const double* src) {
    return scatter_common(c, ptr_kind, fabs, ng, dir, src);
}


int setup_fine_from_faces(mac_ctx* c, const double* fx, const double* fy, const double* fz,
                          const double* alpha_nat, bool reset_flags) {
    Level& L = c->lev[0];
    FineParams P;
    for (int d = 0; d < 3; ++d) {
        P.n[d] = c->n[d];
        P.bc_lo[d] = c->bc_lo[d];
        P.bc_hi[d] = c->bc_hi[d];
        P.active[d] = d < c->dm ? 1 : 0;
        P.ih2[d] = 1.0 / (L.h[d] * L.h[d]);
    }
    P.va = c->va;
    P.p = 0;
    if (reset_flags) MAC_CUDA_TRY(cudaMemsetAsync(c->red.counters, 0, 4 * sizeof(int), c->stream));
    const Grid3 g = grid3(L.d.n0, L.d.n1, L.d.n2);
    k_fine_coef_faces<<<g.grid, g.block, 0, c->stream>>>(
        P, L.d, fx, fy, fz, alpha_nat, alpha_nat ? L.alpha : nullptr, L.a64.bx, L.a64.by,
        L.a64.bz, L.wall[0][0], L.wall[0][1], L.wall[1][0], L.wall[1][1], L.wall[2][0],
        L.wall[2][1]);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    return build_diag(c, 0, mixed(c));
}

int setup_rhs_from(mac_ctx* c, const double* rh_nat, const double* phi_nat) {
    return launch_rhs(c, rh_nat, true, phi_nat);
}

}  // namespace mac
