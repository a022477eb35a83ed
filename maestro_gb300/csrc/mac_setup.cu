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
#include <cstdio>
#include <cstring>

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

__device__ __forceinline__ double beta0_pow(double b, int p) { return p == 2 ? b * b : b; }

// beta' on the low faces of every fine cell, Dirichlet wall planes, density check.
__global__ void __launch_bounds__(kBlock)
k_fine_coef(FineParams P, Dims d, const double* __restrict__ rho, const double* __restrict__ b0,
            const double* __restrict__ b0e, double* __restrict__ bx, double* __restrict__ by,
            double* __restrict__ bz, double* __restrict__ wlo0, double* __restrict__ whi0,
            double* __restrict__ wlo1, double* __restrict__ whi1, double* __restrict__ wlo2,
            double* __restrict__ whi2, int* __restrict__ err) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d.ncell) return;
    const int i = q % P.n[0];
    const int row = q / P.n[0];
    const int j = row % P.n[1];
    const int k = row / P.n[1];
    const int c[3] = {i, j, k};
    const double rc = rho[q];
    if (!(rc > 0.0) || !isfinite(rc)) atomicOr(err, 1);
    const int li = lidx(d, i, j, k);
    double* out[3] = {bx, by, bz};
    double* wl[3] = {wlo0, wlo1, wlo2};
    double* wh[3] = {whi0, whi1, whi2};
    const int r = c[P.va];
#pragma unroll
    for (int dd = 0; dd < 3; ++dd) {
        if (!P.active[dd]) {
            out[dd][li] = 0.0;
            continue;
        }
        const double bcell = P.p ? beta0_pow(b0[r], P.p) : 1.0;
        const double blo = P.p ? (dd == P.va ? beta0_pow(b0e[r], P.p) : bcell) : 1.0;
        double v = 0.0;
        if (c[dd] > 0 || P.bc_lo[dd] == MAC_BC_PER) {
            int nb[3] = {i, j, k};
            nb[dd] = c[dd] > 0 ? c[dd] - 1 : P.n[dd] - 1;
            const double rn = rho[nb[0] + P.n[0] * (nb[1] + P.n[1] * nb[2])];
            v = blo * (2.0 / (rc + rn)) * P.ih2[dd];
        }
        out[dd][li] = v;
        const int plane = dd == 0 ? (j + P.n[1] * k) : dd == 1 ? (i + P.n[0] * k) : (i + P.n[0] * j);
        if (c[dd] == 0 && P.bc_lo[dd] == MAC_BC_DIR)
            wl[dd][plane] = blo * (2.0 / (rc + rc)) * P.ih2[dd];
        if (c[dd] == P.n[dd] - 1 && P.bc_hi[dd] == MAC_BC_DIR) {
            const double bhi = P.p ? (dd == P.va ? beta0_pow(b0e[r + 1], P.p) : bcell) : 1.0;
            wh[dd][plane] = bhi * (2.0 / (rc + rc)) * P.ih2[dd];
        }
    }
}

struct DiagParams {
    int bc_lo[3], bc_hi[3];
    const double* wl[3];
    const double* wh[3];
};

// diag = alpha + sum of the six face coefficients (+ 2 beta'_wall on Dirichlet faces).
__global__ void __launch_bounds__(kBlock)
k_build_diag(Dims d, DiagParams P, const double* __restrict__ bx, const double* __restrict__ by,
             const double* __restrict__ bz, const double* __restrict__ alpha,
             double* __restrict__ dg, double* __restrict__ idg) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d.ncell) return;
    const int i = q % d.n0;
    const int row = q / d.n0;
    const int j = row % d.n1;
    const int k = row / d.n1;
    const int me = lidx(d, i, j, k);
    const int ip = i == d.n0 - 1 ? 0 : i + 1;
    const int jp = j == d.n1 - 1 ? 0 : j + 1;
    const int kp = k == d.n2 - 1 ? 0 : k + 1;
    double s = alpha ? alpha[me] : 0.0;
    s += bx[me] + bx[lidx(d, ip, j, k)];
    s += by[me] + by[lidx(d, i, jp, k)];
    s += bz[me] + bz[lidx(d, i, j, kp)];
    const int c[3] = {i, j, k};
    const int n[3] = {d.n0, d.n1, d.n2};
#pragma unroll
    for (int dd = 0; dd < 3; ++dd) {
        const int plane = dd == 0 ? (j + d.n1 * k) : dd == 1 ? (i + d.n0 * k) : (i + d.n0 * j);
        if (c[dd] == 0 && P.bc_lo[dd] == MAC_BC_DIR && P.wl[dd]) s += 2.0 * P.wl[dd][plane];
        if (c[dd] == n[dd] - 1 && P.bc_hi[dd] == MAC_BC_DIR && P.wh[dd]) s += 2.0 * P.wh[dd][plane];
    }
    dg[me] = s;
    idg[me] = 1.0 / s;
}

// Coarse low-face coefficients: mean of the fine low faces tiling the coarse face, / 4 for h^2.
__global__ void __launch_bounds__(kBlock)
k_coarsen_coef(Dims F, Dims C, const double* __restrict__ fbx, const double* __restrict__ fby,
               const double* __restrict__ fbz, const double* __restrict__ falpha,
               double* __restrict__ cbx, double* __restrict__ cby, double* __restrict__ cbz,
               double* __restrict__ calpha) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= C.ncell) return;
    const int I = q % C.n0;
    const int row = q / C.n0;
    const int J = row % C.n1;
    const int K = row / C.n1;
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
    cbx[me] = 0.25 * sx / (2 * rz);
    cby[me] = 0.25 * sy / (2 * rz);
    cbz[me] = rz == 2 ? 0.25 * sz / 4 : 0.0;
    if (falpha) {
        double sa = 0.0;
        for (int b = 0; b < rz; ++b)
            for (int a1 = 0; a1 < 2; ++a1)
                for (int a0 = 0; a0 < 2; ++a0) sa += falpha[lidx(F, 2 * I + a0, 2 * J + a1, rz * K + b)];
        calpha[me] = sa / (4 * rz);
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
    cw[q] = 0.25 * s / (r0 * r1);
}

__global__ void k_to_f32(int n, const double* __restrict__ a, float* __restrict__ b) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) b[q] = (float)a[q];
}

struct RhsParams {
    int n[3];
    int dm, va, have_beta0;
    double dx[3];
};

// f = -(div(beta0 U) - macrhs) in the level-0 layout, with per-block (sum, max, min).
__global__ void __launch_bounds__(kBlock)
k_rhs(RhsParams P, Dims d, const double* __restrict__ ux, const double* __restrict__ uy,
      const double* __restrict__ uz, const double* __restrict__ macrhs,
      const double* __restrict__ b0, const double* __restrict__ b0e, double* __restrict__ f,
      double* __restrict__ partial) {
    __shared__ double ssum[kBlock], smax[kBlock], smin[kBlock];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0, vmax = -INFINITY, vmin = INFINITY;
    if (q < d.ncell) {
        const int i = q % P.n[0];
        const int row = q / P.n[0];
        const int j = row % P.n[1];
        const int k = row / P.n[1];
        const int c[3] = {i, j, k};
        const double* u[3] = {ux, uy, uz};
        double dv = 0.0;
        for (int dd = 0; dd < P.dm; ++dd) {
            const int m0 = P.n[0] + (dd == 0), m1 = P.n[1] + (dd == 1);
            const int flo = i + m0 * (j + m1 * k);
            const int stride = dd == 0 ? 1 : dd == 1 ? m0 : m0 * m1;
            double ulo = u[dd][flo], uhi = u[dd][flo + stride];
            if (P.have_beta0) {
                const int r = c[P.va];
                if (dd == P.va) {
                    ulo = ulo * b0e[r];
                    uhi = uhi * b0e[r + 1];
                } else {
                    ulo = ulo * b0[r];
                    uhi = uhi * b0[r];
                }
            }
            dv += (uhi - ulo) / P.dx[dd];
        }
        if (macrhs) dv = dv - macrhs[q];
        v = -dv;
        f[lidx(d, i, j, k)] = v;
        vmax = v;
        vmin = v;
    }
    const int t = threadIdx.x;
    ssum[t] = v;
    smax[t] = vmax;
    smin[t] = vmin;
    __syncthreads();
    for (int o = kBlock / 2; o > 0; o >>= 1) {
        if (t < o) {
            ssum[t] += ssum[t + o];
            smax[t] = fmax(smax[t], smax[t + o]);
            smin[t] = fmin(smin[t], smin[t + o]);
            if (isnan(smax[t + o]) || isnan(smax[t])) smax[t] = NAN;
        }
        __syncthreads();
    }
    if (t == 0) {
        partial[3 * blockIdx.x + 0] = ssum[0];
        partial[3 * blockIdx.x + 1] = smax[0];
        partial[3 * blockIdx.x + 2] = smin[0];
    }
}

// Deterministic final reduction of the k_rhs partials: mean and ||f - mean||_inf.
__global__ void k_rhs_final(int nblocks, int ncell, int singular, const double* __restrict__ partial,
                            double* __restrict__ scalars) {
    __shared__ double ssum[1024], smax[1024], smin[1024];
    const int t = threadIdx.x;
    double s = 0.0, mx = -INFINITY, mn = INFINITY;
    bool nan = false;
    for (int b = t; b < nblocks; b += blockDim.x) {
        s += partial[3 * b];
        const double a = partial[3 * b + 1], c = partial[3 * b + 2];
        nan = nan || isnan(a) || isnan(c) || isnan(partial[3 * b]);
        mx = fmax(mx, a);
        mn = fmin(mn, c);
    }
    ssum[t] = s;
    smax[t] = nan ? NAN : mx;
    smin[t] = mn;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (t < o) {
            ssum[t] += ssum[t + o];
            const bool n2 = isnan(smax[t]) || isnan(smax[t + o]);
            smax[t] = n2 ? NAN : fmax(smax[t], smax[t + o]);
            smin[t] = fmin(smin[t], smin[t + o]);
        }
        __syncthreads();
    }
    if (t == 0) {
        const double mean = singular ? ssum[0] / ncell : 0.0;
        scalars[0] = mean;
        scalars[1] = fmax(smax[0] - mean, mean - smin[0]);
        if (isnan(smax[0]) || !isfinite(ssum[0])) scalars[1] = NAN;
        scalars[2] = ssum[0];
        scalars[3] = smax[0];
        scalars[4] = smin[0];
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
    double dx;
    double h2;   // h_dir^2 (beta = beta' * h2)
};

// U = (beta0 U - beta_f G phi) / beta0 on every face normal to P.dir (natural face layout).
__global__ void __launch_bounds__(kBlock)
k_correct(CorrParams P, Dims d, double* __restrict__ u, const double* __restrict__ phi,
          const double* __restrict__ bd, const double* __restrict__ wlo,
          const double* __restrict__ whi, const double* __restrict__ b0,
          const double* __restrict__ b0e) {
    const int m0 = P.n[0] + (P.dir == 0), m1 = P.n[1] + (P.dir == 1), m2 = P.n[2] + (P.dir == 2);
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m0 * m1 * m2) return;
    const int i = q % m0;
    const int row = q / m0;
    const int j = row % m1;
    const int k = row / m1;
    int c[3] = {i, j, k};
    const int dir = P.dir;
    const int nd = P.n[dir];
    const int qd = c[dir];
    double bb = 1.0;
    if (P.have_beta0) {
        const int r = c[P.va];
        bb = (dir == P.va) ? b0e[r] : b0[r];
    }
    double x = u[q];
    if (P.have_beta0) x = x * bb;
    double beta = 0.0, g = 0.0;
    const int plane = dir == 0 ? (j + P.n[1] * k) : dir == 1 ? (i + P.n[0] * k) : (i + P.n[0] * j);
    if (qd > 0 && qd < nd) {
        int lo[3] = {c[0], c[1], c[2]};
        lo[dir] -= 1;
        const int chi = lidx(d, c[0], c[1], c[2]);
        beta = bd[chi] * P.h2;
        g = (phi[chi] - phi[lidx(d, lo[0], lo[1], lo[2])]) / P.dx;
    } else if ((qd == 0 && P.bc_lo == MAC_BC_PER) || (qd == nd && P.bc_hi == MAC_BC_PER)) {
        int hi[3] = {c[0], c[1], c[2]}, lo[3] = {c[0], c[1], c[2]};
        hi[dir] = 0;
        lo[dir] = nd - 1;
        const int chi = lidx(d, hi[0], hi[1], hi[2]);
        beta = bd[chi] * P.h2;
        g = (phi[chi] - phi[lidx(d, lo[0], lo[1], lo[2])]) / P.dx;
    } else if (qd == 0) {
        if (P.bc_lo == MAC_BC_DIR) {
            beta = wlo[plane] * P.h2;
            g = 2.0 * phi[lidx(d, c[0], c[1], c[2])] / P.dx;
        }
    } else {
        if (P.bc_hi == MAC_BC_DIR) {
            int lo[3] = {c[0], c[1], c[2]};
            lo[dir] -= 1;
            beta = whi[plane] * P.h2;
            g = -2.0 * phi[lidx(d, lo[0], lo[1], lo[2])] / P.dx;
        }
    }
    x = x - beta * g;
    if (P.have_beta0) x = x / bb;
    u[q] = x;
}

__global__ void k_nat_to_l0(Dims d, const double* __restrict__ src, double* __restrict__ dst) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d.ncell) return;
    const int i = q % d.n0, row = q / d.n0, j = row % d.n1, k = row / d.n1;
    dst[lidx(d, i, j, k)] = src[q];
}

__global__ void k_l0_to_nat(Dims d, const double* __restrict__ src, double* __restrict__ dst) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d.ncell) return;
    const int i = q % d.n0, row = q / d.n0, j = row % d.n1, k = row / d.n1;
    dst[q] = src[lidx(d, i, j, k)];
}

// ---- caller box layout <-> whole-domain natural arrays --------------------------------------
struct GatherParams {
    int n[3];       // domain cells (internal 3-D)
    int dm;
    int dir;        // -1: cell field; 0..2: faces normal to dir
    int bc_per[3];  // periodic flag per direction
};

// Whole-domain array <- valid region of every box.  Faces: each box writes lo..hi along dir,
// and hi+1 only at the domain's high end.
__global__ void k_gather(GatherParams P, const BoxDesc* __restrict__ boxes, double* __restrict__ dst) {
    const BoxDesc B = boxes[blockIdx.y];
    const int e0 = B.hi[0] - B.lo[0] + 1 + (P.dir == 0);
    const int e1 = B.hi[1] - B.lo[1] + 1 + (P.dir == 1);
    const int e2 = B.hi[2] - B.lo[2] + 1 + (P.dir == 2);
    const int m0 = P.n[0] + (P.dir == 0), m1 = P.n[1] + (P.dir == 1);
    const int total = e0 * e1 * e2;
    const int g0 = B.ng, g1 = B.ng, g2 = P.dm == 3 ? B.ng : 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int a = t % e0, row = t / e0, b = row % e1, c = row / e1;
        const int gi = B.lo[0] + a, gj = B.lo[1] + b, gk = B.lo[2] + c;
        if (P.dir >= 0) {
            const int gc[3] = {gi, gj, gk};
            const int hi = (P.dir == 0 ? B.hi[0] : P.dir == 1 ? B.hi[1] : B.hi[2]);
            if (gc[P.dir] == hi + 1 && hi + 1 != P.n[P.dir]) continue;
        }
        const long src = (long)(a + g0) + (long)B.ext[0] * ((b + g1) + (long)B.ext[1] * (c + g2));
        dst[gi + (long)m0 * (gj + (long)m1 * gk)] = B.ptr[B.comp_off + src];
    }
}

// Every entry of every fab (valid + ghosts) <- whole-domain array, periodic wrap; ghosts outside
// a non-periodic domain boundary are left untouched.
__global__ void k_scatter(GatherParams P, const BoxDesc* __restrict__ boxes,
                          const double* __restrict__ src) {
    const BoxDesc B = boxes[blockIdx.y];
    double* dst = const_cast<double*>(B.ptr);
    const int total = B.ext[0] * B.ext[1] * B.ext[2];
    const int m0 = P.n[0] + (P.dir == 0), m1 = P.n[1] + (P.dir == 1);
    const int g[3] = {B.ng, B.ng, P.dm == 3 ? B.ng : 0};
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int a = t % B.ext[0], row = t / B.ext[0], b = row % B.ext[1], c = row / B.ext[1];
        int gc[3] = {B.lo[0] - g[0] + a, B.lo[1] - g[1] + b, B.lo[2] - g[2] + c};
        bool ok = true;
        for (int dd = 0; dd < 3; ++dd) {
            const int lim = P.n[dd] + (P.dir == dd ? 1 : 0);
            if (gc[dd] < 0 || gc[dd] >= lim) {
                if (!P.bc_per[dd]) {
                    ok = false;
                    break;
                }
                gc[dd] = (gc[dd] % P.n[dd] + P.n[dd]) % P.n[dd];
            }
        }
        if (!ok) continue;
        dst[t] = src[gc[0] + (long)m0 * (gc[1] + (long)m1 * gc[2])];
    }
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
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d.ncell) return;
    const int i = q % P.n[0];
    const int row = q / P.n[0];
    const int j = row % P.n[1];
    const int k = row / P.n[1];
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

// f <- rh (natural) in the level-0 layout, with the per-block (sum, max, min) of k_rhs.
__global__ void __launch_bounds__(kBlock)
k_load_rhs(Dims d, const double* __restrict__ rh, double* __restrict__ f,
           double* __restrict__ partial) {
    __shared__ double ssum[kBlock], smax[kBlock], smin[kBlock];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0, vmax = -INFINITY, vmin = INFINITY;
    if (q < d.ncell) {
        const int i = q % d.n0, row = q / d.n0, j = row % d.n1, k = row / d.n1;
        v = rh[q];
        f[lidx(d, i, j, k)] = v;
        vmax = v;
        vmin = v;
    }
    const int t = threadIdx.x;
    ssum[t] = v;
    smax[t] = vmax;
    smin[t] = vmin;
    __syncthreads();
    for (int o = kBlock / 2; o > 0; o >>= 1) {
        if (t < o) {
            ssum[t] += ssum[t + o];
            const bool n2 = isnan(smax[t]) || isnan(smax[t + o]);
            smax[t] = n2 ? NAN : fmax(smax[t], smax[t + o]);
            smin[t] = fmin(smin[t], smin[t + o]);
        }
        __syncthreads();
    }
    if (t == 0) {
        partial[3 * blockIdx.x + 0] = ssum[0];
        partial[3 * blockIdx.x + 1] = smax[0];
        partial[3 * blockIdx.x + 2] = smin[0];
    }
}

Dims level0_dims(const mac_ctx* c) { return c->lev[0].d; }

}  // namespace

// ------------------------------------------------------------------------------------------
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
    k_fine_coef<<<ceil_div(L.d.ncell, kBlock), kBlock, 0, c->stream>>>(
        P, L.d, c->rho, beta0, beta0e, L.a64.bx, L.a64.by, L.a64.bz, L.wall[0][0], L.wall[0][1],
        L.wall[1][0], L.wall[1][1], L.wall[2][0], L.wall[2][1], c->red.counters + 1);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    DiagParams D;
    for (int d = 0; d < 3; ++d) {
        D.bc_lo[d] = c->bc_lo[d];
        D.bc_hi[d] = c->bc_hi[d];
        D.wl[d] = L.wall[d][0];
        D.wh[d] = L.wall[d][1];
    }
    k_build_diag<<<ceil_div(L.d.ncell, kBlock), kBlock, 0, c->stream>>>(
        L.d, D, L.a64.bx, L.a64.by, L.a64.bz, L.alpha, L.a64.diag, L.a64.invdiag);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    return MAC_OK;
}

int setup_coarse_levels(mac_ctx* c) {
    for (int l = 1; l < c->nlevels; ++l) {
        Level& F = c->lev[l - 1];
        Level& C = c->lev[l];
        k_coarsen_coef<<<ceil_div(C.d.ncell, kBlock), kBlock, 0, c->stream>>>(
            F.d, C.d, F.a64.bx, F.a64.by, F.a64.bz, F.alpha, C.a64.bx, C.a64.by, C.a64.bz, C.alpha);
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
        DiagParams D;
        for (int d = 0; d < 3; ++d) {
            D.bc_lo[d] = c->bc_lo[d];
            D.bc_hi[d] = c->bc_hi[d];
            D.wl[d] = C.wall[d][0];
            D.wh[d] = C.wall[d][1];
        }
        k_build_diag<<<ceil_div(C.d.ncell, kBlock), kBlock, 0, c->stream>>>(
            C.d, D, C.a64.bx, C.a64.by, C.a64.bz, C.alpha, C.a64.diag, C.a64.invdiag);
        MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    }
    return MAC_OK;
}

int setup_fp32_copies(mac_ctx* c) {
    for (int l = 0; l < c->nlevels; ++l) {
        Level& L = c->lev[l];
        if (!L.a32.bx) continue;
        const int n = L.d.ncell;
        const double* src[5] = {L.a64.bx, L.a64.by, L.a64.bz, L.a64.diag, L.a64.invdiag};
        float* dst[5] = {L.a32.bx, L.a32.by, L.a32.bz, L.a32.diag, L.a32.invdiag};
        for (int a = 0; a < 5; ++a) {
            k_to_f32<<<ceil_div(n, kBlock), kBlock, 0, c->stream>>>(n, src[a], dst[a]);
            MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
        }
    }
    return MAC_OK;
}

int setup_rhs(mac_ctx* c, const double* macrhs, bool have_beta0) {
    Level& L = c->lev[0];
    RhsParams P;
    for (int d = 0; d < 3; ++d) {
        P.n[d] = c->n[d];
        P.dx[d] = c->dx[d];
    }
    P.dm = c->dm;
    P.va = c->va;
    P.have_beta0 = have_beta0 ? 1 : 0;
    const int nb = ceil_div(L.d.ncell, kBlock);
    k_rhs<<<nb, kBlock, 0, c->stream>>>(P, L.d, c->u[0], c->u[1], c->u[2], macrhs, c->beta0,
                                        c->beta0e, L.a64.f, c->red.partial);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    k_rhs_final<<<1, 1024, 0, c->stream>>>(nb, L.d.ncell, c->singular ? 1 : 0, c->red.partial,
                                           c->red.scalars);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    if (c->singular) {
        k_sub_mean<<<nb, kBlock, 0, c->stream>>>(L.d.ncell, L.a64.f, c->red.scalars);
        MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    }
    return MAC_OK;
}

int correct_velocity(mac_ctx* c, bool have_beta0) {
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
        P.dx = c->dx[d];
        P.h2 = c->dx[d] * c->dx[d];
        const long nf = (long)(c->n[0] + (d == 0)) * (c->n[1] + (d == 1)) * (c->n[2] + (d == 2));
        k_correct<<<ceil_div(nf, kBlock), kBlock, 0, c->stream>>>(
            P, L.d, c->u[d], L.a64.phi, bd[d], L.wall[d][0], L.wall[d][1], c->beta0, c->beta0e);
        MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    }
    return MAC_OK;
}

int natural_to_level0(mac_ctx* c, const double* src, double* dst) {
    const Dims d = level0_dims(c);
    k_nat_to_l0<<<ceil_div(d.ncell, kBlock), kBlock, 0, c->stream>>>(d, src, dst);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    return MAC_OK;
}

int level0_to_natural(mac_ctx* c, const double* src, double* dst) {
    const Dims d = level0_dims(c);
    k_l0_to_nat<<<ceil_div(d.ncell, kBlock), kBlock, 0, c->stream>>>(d, src, dst);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    return MAC_OK;
}

// ---- box tables ----------------------------------------------------------------------------
namespace {

constexpr int kBoxSlots = 16;

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
    MAC_CUDA_TRY(cudaMemcpyAsync(d, h, sizeof(BoxDesc) * nb, cudaMemcpyHostToDevice, c->stream));
    *dev_table = d;
    return MAC_OK;
}

int ensure_staging(mac_ctx* c, size_t elems) {
    if (elems <= c->staging_elems) return MAC_OK;
    if (c->staging) {
        MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
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

size_t host_staging_need(const mac_ctx* c, int dir, int ng) {
    size_t tot = 0;
    for (int b = 0; b < c->g.nboxes; ++b) {
        size_t e = 1;
        for (int d = 0; d < 3; ++d) {
            const int g = d < c->dm ? ng : 0;
            const int lo = d < c->dm ? c->box_lo[3 * b + d] : 0;
            const int hi = d < c->dm ? c->box_hi[3 * b + d] : 0;
            e *= (size_t)(hi - lo + 1 + (dir == d ? 1 : 0) + 2 * g);
        }
        tot += e;
    }
    return tot;
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

int gather_common(mac_ctx* c, int ptr_kind, const double* const* fabs, int ng, int ncomp, int comp,
                  int dir, double* dst) {
    if (ptr_kind == MAC_PTR_HOST) {
        int rc = ensure_staging(c, host_staging_need(c, dir, ng));
        if (rc) return rc;
    }
    BoxDesc* table = nullptr;
    size_t tot = 0;
    std::vector<size_t> offs;
    int rc = fill_boxes(c, dir, ng, ncomp, comp, fabs, ptr_kind, true, &table, &tot, &offs);
    if (rc) return rc;
    if (ptr_kind == MAC_PTR_HOST) {
        for (int b = 0; b < c->g.nboxes; ++b) {
            const BoxDesc& B = c->h_boxes[0];
            (void)B;
            size_t e = 1;
            for (int d = 0; d < 3; ++d) {
                const int g = d < c->dm ? ng : 0;
                const int lo = d < c->dm ? c->box_lo[3 * b + d] : 0;
                const int hi = d < c->dm ? c->box_hi[3 * b + d] : 0;
                e *= (size_t)(hi - lo + 1 + (dir == d ? 1 : 0) + 2 * g);
            }
            MAC_CUDA_TRY(cudaMemcpyAsync(c->staging + offs[b], fabs[b] + e * comp, e * sizeof(double),
                                         cudaMemcpyHostToDevice, c->stream));
        }
    }
    const GatherParams P = gparams(c, dir);
    dim3 grid(64, c->g.nboxes);
    k_gather<<<grid, kBlock, 0, c->stream>>>(P, table, dst);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    if (ptr_kind == MAC_PTR_HOST) MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MAC_OK;
}

int scatter_common(mac_ctx* c, int ptr_kind, double* const* fabs, int ng, int dir,
                   const double* src) {
    if (ptr_kind == MAC_PTR_HOST) {
        int rc = ensure_staging(c, host_staging_need(c, dir, ng));
        if (rc) return rc;
    }
    BoxDesc* table = nullptr;
    size_t tot = 0;
    std::vector<size_t> offs;
    int rc = fill_boxes(c, dir, ng, 1, 0, (const double* const*)fabs, ptr_kind, true, &table, &tot,
                        &offs);
    if (rc) return rc;
    if (ptr_kind == MAC_PTR_HOST) {
        // the kernel writes every fab entry it can; copy the current host contents first so the
        // entries it leaves alone (physical-boundary ghosts) survive the round trip
        for (int b = 0; b < c->g.nboxes; ++b) {
            size_t e = 1;
            for (int d = 0; d < 3; ++d) {
                const int g = d < c->dm ? ng : 0;
                const int lo = d < c->dm ? c->box_lo[3 * b + d] : 0;
                const int hi = d < c->dm ? c->box_hi[3 * b + d] : 0;
                e *= (size_t)(hi - lo + 1 + (dir == d ? 1 : 0) + 2 * g);
            }
            MAC_CUDA_TRY(cudaMemcpyAsync(c->staging + offs[b], fabs[b], e * sizeof(double),
                                         cudaMemcpyHostToDevice, c->stream));
        }
    }
    const GatherParams P = gparams(c, dir);
    dim3 grid(64, c->g.nboxes);
    k_scatter<<<grid, kBlock, 0, c->stream>>>(P, table, src);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    if (ptr_kind == MAC_PTR_HOST) {
        for (int b = 0; b < c->g.nboxes; ++b) {
            size_t e = 1;
            for (int d = 0; d < 3; ++d) {
                const int g = d < c->dm ? ng : 0;
                const int lo = d < c->dm ? c->box_lo[3 * b + d] : 0;
                const int hi = d < c->dm ? c->box_hi[3 * b + d] : 0;
                e *= (size_t)(hi - lo + 1 + (dir == d ? 1 : 0) + 2 * g);
            }
            MAC_CUDA_TRY(cudaMemcpyAsync(fabs[b], c->staging + offs[b], e * sizeof(double),
                                         cudaMemcpyDeviceToHost, c->stream));
        }
        MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
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
                          const double* alpha_nat) {
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
    MAC_CUDA_TRY(cudaMemsetAsync(c->red.counters, 0, 4 * sizeof(int), c->stream));
    k_fine_coef_faces<<<ceil_div(L.d.ncell, kBlock), kBlock, 0, c->stream>>>(
        P, L.d, fx, fy, fz, alpha_nat, alpha_nat ? L.alpha : nullptr, L.a64.bx, L.a64.by,
        L.a64.bz, L.wall[0][0], L.wall[0][1], L.wall[1][0], L.wall[1][1], L.wall[2][0],
        L.wall[2][1]);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    DiagParams D;
    for (int d = 0; d < 3; ++d) {
        D.bc_lo[d] = c->bc_lo[d];
        D.bc_hi[d] = c->bc_hi[d];
        D.wl[d] = L.wall[d][0];
        D.wh[d] = L.wall[d][1];
    }
    k_build_diag<<<ceil_div(L.d.ncell, kBlock), kBlock, 0, c->stream>>>(
        L.d, D, L.a64.bx, L.a64.by, L.a64.bz, alpha_nat ? L.alpha : nullptr, L.a64.diag,
        L.a64.invdiag);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    return MAC_OK;
}

int setup_rhs_from(mac_ctx* c, const double* rh_nat) {
    Level& L = c->lev[0];
    const int nb = ceil_div(L.d.ncell, kBlock);
    k_load_rhs<<<nb, kBlock, 0, c->stream>>>(L.d, rh_nat, L.a64.f, c->red.partial);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    k_rhs_final<<<1, 1024, 0, c->stream>>>(nb, L.d.ncell, c->singular ? 1 : 0, c->red.partial,
                                           c->red.scalars);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    if (c->singular) {
        k_sub_mean<<<nb, kBlock, 0, c->stream>>>(L.d.ncell, L.a64.f, c->red.scalars);
        MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    }
    return MAC_OK;
}

}  // namespace mac
