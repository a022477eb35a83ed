// Adjoint (reverse-mode derivative) of the whole-domain MAC projection.  No counterpart in the
// reference; the forward map is the one of Source/macproject.f90:51-328 as implemented here.
//
// Forward (entries e of the face arrays; face 0 and face n of a periodic direction are separate
// entries of the same physical face):
//   h_f     = 2 / (rho_a + rho_b)                   (physical face f between cells a, b)
//   beta_f  = beta0_f^p h_f,   c_e = beta0_e^(p-1) h_f(e),   p = 1 (+1 with use_alt_energy_fix)
//   f       = P (macrhs - D(beta0 U))               (P removes the mean: singular problem)
//   L phi   = G^T B G phi = f                       (G: cells -> physical faces, 0 on walls)
//   U_proj  = U - c (G phi)
// Loss L = sum_e w_e U_proj,e.  Reverse sweep:
//   lambda  = dL/dphi = G^T-weighted sum of c_e w_e        (k_adj_rhs)
//   L mu    = lambda   -- the same V-cycle solves it (L is symmetric), nu = P mu
//   dL/dmacrhs = nu
//   dL/dU_e    = w_e + beta0_e (nu_hi - nu_lo)/dx   (zero outside the domain: D^T per entry)
//   dL/dbeta_f = -(G nu)_f (G phi)_f,   dL/dc_e = -w_e (G phi)_e
//   dL/dh_f    = beta0^p dL/dbeta_f + sum_{e on f} beta0_e^(p-1) dL/dc_e
//   dL/d(1/rho_a) = sum_{f of a} dL/dh_f * h_f^2 rho_a^2 / 2
//   dL/dbeta0_e   = -U_e (D^T nu)_e + p beta0^(p-1) h dL/dbeta_f + (p-1) beta0^(p-2) h dL/dc_e,
//   summed per layer, beta0_edge = cell_to_edge(beta0) chained on the host (1-D).
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "mac_internal.cuh"

namespace mac {
namespace {

constexpr int kB = 256;

struct AdjGeom {
    int n[3];
    int dm, va, p;
    int per[3];
    double idx[3];
    Dims d0;
};

__device__ __forceinline__ double ipow(double b, int e) {
    return e == 0 ? 1.0 : (e == 1 ? b : b * b);
}

__device__ __forceinline__ int nat(const AdjGeom& G, int i, int j, int k) {
    return i + G.n[0] * (j + G.n[1] * k);
}

__device__ __forceinline__ int face_nat(const AdjGeom& G, int d, int i, int j, int k) {
    const int m0 = G.n[0] + (d == 0), m1 = G.n[1] + (d == 1);
    return i + m0 * (j + m1 * k);
}

// beta0 on a face entry of direction d whose cell/face coordinate along the vertical is r.
__device__ __forceinline__ double b0_face(const AdjGeom& G, const double* b0, const double* b0e,
                                          int d, int r) {
    if (G.p == 0) return 1.0;
    return d == G.va ? b0e[r] : b0[r];
}

// lambda_a = sum over the face entries touching cell a of c_e w_e (+1/dx on the low entry,
// -1/dx on the high entry), walls excluded.
__global__ void __launch_bounds__(kB)
k_adj_rhs(AdjGeom G, const double* __restrict__ rho, const double* __restrict__ b0,
          const double* __restrict__ b0e, const double* __restrict__ wx,
          const double* __restrict__ wy, const double* __restrict__ wz,
          double* __restrict__ lam) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= G.d0.ncell) return;
    const int i = q % G.n[0], row = q / G.n[0], j = row % G.n[1], k = row / G.n[1];
    const int c[3] = {i, j, k};
    const double* w[3] = {wx, wy, wz};
    const double rc = rho[q];
    double s = 0.0;
    for (int d = 0; d < G.dm; ++d) {
        const int n = G.n[d];
        // low physical face
        if (c[d] > 0 || G.per[d]) {
            int nb[3] = {i, j, k};
            nb[d] = c[d] > 0 ? c[d] - 1 : n - 1;
            const double h = 2.0 / (rc + rho[nat(G, nb[0], nb[1], nb[2])]);
            int e[3] = {i, j, k};
            double wl = w[d][face_nat(G, d, e[0], e[1], e[2])];
            if (c[d] == 0) {   // periodic: entry n is the same physical face
                e[d] = n;
                wl += w[d][face_nat(G, d, e[0], e[1], e[2])];
            }
            const int r = d == G.va ? c[G.va] : c[G.va];
            const double cc = ipow(b0_face(G, b0, b0e, d, r), G.p > 0 ? G.p - 1 : 0) * h;
            s -= cc * wl * G.idx[d];
        }
        // high physical face
        if (c[d] < n - 1 || G.per[d]) {
            int nb[3] = {i, j, k};
            nb[d] = c[d] < n - 1 ? c[d] + 1 : 0;
            const double h = 2.0 / (rc + rho[nat(G, nb[0], nb[1], nb[2])]);
            int e[3] = {i, j, k};
            e[d] = c[d] + 1;
            double wh = w[d][face_nat(G, d, e[0], e[1], e[2])];
            if (c[d] == n - 1) {   // periodic: entry 0 is the same physical face
                e[d] = 0;
                wh += w[d][face_nat(G, d, e[0], e[1], e[2])];
            }
            const int r = d == G.va ? c[G.va] + 1 : c[G.va];
            const double cc = ipow(b0_face(G, b0, b0e, d, r), G.p > 0 ? G.p - 1 : 0) * h;
            s += cc * wh * G.idx[d];
        }
    }
    lam[q] = s;
}

// Deterministic block partial sums of a level-0 array (for the mean of mu).
__global__ void __launch_bounds__(kB)
k_partial_sum(int n, const double* __restrict__ a, double* __restrict__ part) {
    __shared__ double sm[kB];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    sm[threadIdx.x] = q < n ? a[q] : 0.0;
    __syncthreads();
    for (int o = kB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

__global__ void k_final_mean(int nb, int n, const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sm[1024];
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[b];
    sm[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = sm[0] / n;
}

struct FaceOut {
    double* du;     // dL/dU entries (natural face layout)
    double* dh;     // per-entry share of dL/dh_f
    double* db0;    // per-entry dL/dbeta0_e
};

// Per face entry of direction d: dU, dh share, dbeta0 share.
__global__ void __launch_bounds__(kB)
k_adj_face(AdjGeom G, int d, const double* __restrict__ rho, const double* __restrict__ b0,
           const double* __restrict__ b0e, const double* __restrict__ u,
           const double* __restrict__ w, const double* __restrict__ phi,
           const double* __restrict__ mu, const double* __restrict__ mean_mu, FaceOut out) {
    const int m0 = G.n[0] + (d == 0), m1 = G.n[1] + (d == 1), m2 = G.n[2] + (d == 2);
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m0 * m1 * m2) return;
    const int i = q % m0, row = q / m0, j = row % m1, k = row / m1;
    const int f[3] = {i, j, k};
    const int n = G.n[d];
    const int qd = f[d];
    const double mm = *mean_mu;
    const double dx1 = G.idx[d];
    // cells on either side (may be outside the domain)
    int lo[3] = {i, j, k}, hi[3] = {i, j, k};
    lo[d] = qd - 1;
    const bool lo_in = qd > 0, hi_in = qd < n;
    // -(D^T nu)_e = (nu_hi - nu_lo)/dx with nu = 0 outside the domain
    const double nu_hi = hi_in ? mu[level_index(G.d0, hi[0], hi[1], hi[2])] - mm : 0.0;
    const double nu_lo = lo_in ? mu[level_index(G.d0, lo[0], lo[1], lo[2])] - mm : 0.0;
    const double dtnu = (nu_hi - nu_lo) * dx1;
    const int r = d == G.va ? qd : f[G.va];
    const double bb = b0_face(G, b0, b0e, d, r);
    const double ue = u[q], we = w[q];
    double du = we + bb * dtnu;
    double dh = 0.0, db0 = u[q] * dtnu;
    // physical face: interior, or a periodic boundary entry (0 or n)
    const bool interior = qd > 0 && qd < n;
    const bool per_entry = G.per[d] && (qd == 0 || qd == n);
    if (interior || per_entry) {
        int a[3] = {i, j, k}, b[3] = {i, j, k};
        a[d] = interior ? qd - 1 : n - 1;
        b[d] = interior ? qd : 0;
        const int ia = level_index(G.d0, a[0], a[1], a[2]);
        const int ib = level_index(G.d0, b[0], b[1], b[2]);
        const double gphi = (phi[ib] - phi[ia]) * dx1;
        const double gnu = (mu[ib] - mu[ia]) * dx1;
        const double h = 2.0 / (rho[nat(G, a[0], a[1], a[2])] + rho[nat(G, b[0], b[1], b[2])]);
        const double dc = -we * gphi;
        // the solve uses each physical face once: entry n of a periodic direction is the duplicate
        const double dbeta = (qd == n) ? 0.0 : -gnu * gphi;
        const int p = G.p > 0 ? G.p : 1;
        dh = ipow(bb, p) * dbeta + ipow(bb, p - 1) * dc;
        if (G.p > 0) db0 += p * ipow(bb, p - 1) * h * dbeta + (p - 1) * h * dc;
    }
    (void)ue;
    out.du[q] = du;
    out.dh[q] = dh;
    out.db0[q] = db0;
}

// dL/d(1/rho_a) = sum over the physical faces of a of dL/dh_f * h_f^2 rho_a^2 / 2.
__global__ void __launch_bounds__(kB)
k_adj_sigma(AdjGeom G, const double* __restrict__ rho, const double* __restrict__ dhx,
            const double* __restrict__ dhy, const double* __restrict__ dhz,
            double* __restrict__ ds) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= G.d0.ncell) return;
    const int i = q % G.n[0], row = q / G.n[0], j = row % G.n[1], k = row / G.n[1];
    const int c[3] = {i, j, k};
    const double* dh[3] = {dhx, dhy, dhz};
    const double rc = rho[q];
    double s = 0.0;
    for (int d = 0; d < G.dm; ++d) {
        const int n = G.n[d];
        if (c[d] > 0 || G.per[d]) {
            int nb[3] = {i, j, k};
            nb[d] = c[d] > 0 ? c[d] - 1 : n - 1;
            const double h = 2.0 / (rc + rho[nat(G, nb[0], nb[1], nb[2])]);
            int e[3] = {i, j, k};
            double g = dh[d][face_nat(G, d, e[0], e[1], e[2])];
            if (c[d] == 0) {
                e[d] = n;
                g += dh[d][face_nat(G, d, e[0], e[1], e[2])];
            }
            s += g * h * h;
        }
        if (c[d] < n - 1 || G.per[d]) {
            int nb[3] = {i, j, k};
            nb[d] = c[d] < n - 1 ? c[d] + 1 : 0;
            const double h = 2.0 / (rc + rho[nat(G, nb[0], nb[1], nb[2])]);
            int e[3] = {i, j, k};
            e[d] = c[d] + 1;
            double g = dh[d][face_nat(G, d, e[0], e[1], e[2])];
            if (c[d] == n - 1) {
                e[d] = 0;
                g += dh[d][face_nat(G, d, e[0], e[1], e[2])];
            }
            s += g * h * h;
        }
    }
    ds[q] = s * rc * rc * 0.5;
}

// One CTA per vertical index r: sum of the per-entry dbeta0 shares of the horizontal faces in
// layer r (r < nr) into sh[r], of the vertical faces in plane r (r <= nr) into sv[r].
__global__ void __launch_bounds__(kB)
k_layer_sums(AdjGeom G, const double* __restrict__ bx, const double* __restrict__ by,
             const double* __restrict__ bz, double* __restrict__ sh, double* __restrict__ sv) {
    __shared__ double s1[kB], s2[kB];
    const int r = blockIdx.x;
    const int nr = G.n[G.va];
    const double* b[3] = {bx, by, bz};
    double a = 0.0, v = 0.0;
    for (int d = 0; d < G.dm; ++d) {
        const int m[3] = {G.n[0] + (d == 0), G.n[1] + (d == 1), G.n[2] + (d == 2)};
        if (d == G.va && r > nr) continue;
        if (d != G.va && r >= nr) continue;
        // entries with vertical coordinate r: iterate over the other two directions
        const int o0 = G.va == 0 ? 1 : 0, o1 = G.va == 2 ? 1 : 2;
        const int cnt = m[o0] * m[o1];
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
            int e[3];
            e[o0] = t % m[o0];
            e[o1] = t / m[o0];
            e[G.va] = r;
            const double x = b[d][e[0] + m[0] * (e[1] + m[1] * e[2])];
            if (d == G.va) v += x;
            else a += x;
        }
    }
    s1[threadIdx.x] = a;
    s2[threadIdx.x] = v;
    __syncthreads();
    for (int o = kB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            s1[threadIdx.x] += s1[threadIdx.x + o];
            s2[threadIdx.x] += s2[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (r < nr) sh[r] = s1[0];
        sv[r] = s2[0];
    }
}

__global__ void k_mu_to_nat(Dims d, const double* __restrict__ mu, const double* __restrict__ mean,
                            double* __restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d.ncell) return;
    const int i = q % d.n0, row = q / d.n0, j = row % d.n1, k = row / d.n1;
    out[q] = mu[level_index(d, i, j, k)] - mean[0];
}

// Transpose of cell_to_edge (Source/cell_to_edge.f90:39-60) applied to the edge sensitivities sv:
// adds sum_r sv[r] d(edge_r)/d(cell_k) to g[k].  The limiter is taken in the branch the forward
// evaluation selects.
void cell_to_edge_vjp(int nr, const double* c, const double* sv, double* g) {
    for (int r = 0; r <= nr; ++r) {
        const double s = sv[r];
        if (r == 0) {
            g[0] += s;
        } else if (r == 1) {
            g[0] += 0.5 * s;
            if (nr > 1) g[1] += 0.5 * s;
        } else if (r == nr) {
            g[r - 1] += s;
        } else if (r == nr - 1) {
            g[r] += 0.5 * s;
            g[r - 1] += 0.5 * s;
        } else {
            const double tmp = 7.0 / 12.0 * (c[r] + c[r - 1]) - 1.0 / 12.0 * (c[r + 1] + c[r - 2]);
            const double lo = std::min(c[r], c[r - 1]), hi = std::max(c[r], c[r - 1]);
            if (tmp < lo) {
                g[c[r] <= c[r - 1] ? r : r - 1] += s;
            } else if (tmp > hi) {
                g[c[r] >= c[r - 1] ? r : r - 1] += s;
            } else {
                g[r] += 7.0 / 12.0 * s;
                g[r - 1] += 7.0 / 12.0 * s;
                g[r + 1] -= 1.0 / 12.0 * s;
                g[r - 2] -= 1.0 / 12.0 * s;
            }
        }
    }
}

struct AdjBuffers {
    double* phiF = nullptr;     // forward phi, level-0 layout
    double* part = nullptr;     // partial sums
    double* mean = nullptr;     // [1]
    double* dh[3] = {nullptr, nullptr, nullptr};
    double* db0[3] = {nullptr, nullptr, nullptr};
    double* layer = nullptr;    // sh[nr], sv[nr+1]
    bool ready = false;
};

}  // namespace
}  // namespace mac

using namespace mac;

extern "C" int mac_macproject_adjoint_dense(mac_ctx* c, const double* ux, const double* uy,
                                            const double* uz, const double* rho,
                                            const double* macrhs, const double* beta0,
                                            const double* beta0_edge, const double* wx,
                                            const double* wy, const double* wz, double* dux,
                                            double* duy, double* duz, double* drinv,
                                            double* dbeta0, double* dmacrhs, double* phi_out,
                                            mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if (!c || !ux || !uy || !rho || !wx || !wy || !dux || !duy) return st->status = MAC_ERR_INVALID;
    if (c->dm == 3 && (!uz || !wz || !duz)) return st->status = MAC_ERR_INVALID;
    if ((beta0 == nullptr) != (beta0_edge == nullptr)) return st->status = MAC_ERR_INVALID;
    if (dbeta0 && !beta0) return st->status = MAC_ERR_INVALID;
    // MAESTRO's vertical direction is never periodic (beta0 is a stratified profile); the
    // periodic-vertical face bookkeeping of beta0_edge is not differentiated
    if (beta0 && c->bc_lo[c->va] == MAC_BC_PER) return st->status = MAC_ERR_UNSUPPORTED;
    for (int d = 0; d < c->dm; ++d)
        if (c->bc_lo[d] == MAC_BC_DIR || c->bc_hi[d] == MAC_BC_DIR) return st->status = MAC_ERR_UNSUPPORTED;
    const auto t0 = std::chrono::steady_clock::now();
    begin_call_stats(c, st);
    // adjoint buffers live with the context's allocations (freed by mac_ctx_destroy)
    const size_t N = (size_t)c->n[0] * c->n[1] * c->n[2];
    const int nr = c->n[c->va];
    const int nbp = ceil_div((long)N, kB);
    AdjBuffers B;
    int rc = MAC_OK;
    rc |= alloc_device(c, (void**)&B.phiF, N * sizeof(double));
    rc |= alloc_device(c, (void**)&B.part, (size_t)nbp * sizeof(double));
    rc |= alloc_device(c, (void**)&B.mean, sizeof(double));
    rc |= alloc_device(c, (void**)&B.layer, (size_t)(2 * nr + 2) * sizeof(double));
    for (int d = 0; d < c->dm; ++d) {
        const size_t nf = (size_t)(c->n[0] + (d == 0)) * (c->n[1] + (d == 1)) * (c->n[2] + (d == 2));
        rc |= alloc_device(c, (void**)&B.dh[d], nf * sizeof(double));
        rc |= alloc_device(c, (void**)&B.db0[d], nf * sizeof(double));
    }
    if (rc) return st->status = MAC_ERR_ALLOC;
    cudaStream_t s = c->stream;
    Level& F = c->lev[0];
    const double* uin[3] = {ux, uy, uz};
    const double* win[3] = {wx, wy, wz};
    double* dout[3] = {dux, duy, duz};
    // ---- forward: phi of the projection (U copied; the caller's arrays stay untouched)
    for (int d = 0; d < c->dm; ++d) {
        const size_t nf = (size_t)(c->n[0] + (d == 0)) * (c->n[1] + (d == 1)) * (c->n[2] + (d == 2));
        MAC_CUDA_TRY(cudaMemcpyAsync(c->u[d], uin[d], nf * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    double* saved_rho = c->rho;
    c->rho = const_cast<double*>(rho);
    MAC_CUDA_TRY(cudaMemsetAsync(c->phin, 0, N * sizeof(double), s));
    if (beta0) rc = load_beta0(c, MAC_PTR_DEVICE, beta0, beta0_edge);
    mac_stats fst;
    std::memset(&fst, 0, sizeof(fst));
    if (!rc) rc = forward_projection(c, macrhs, beta0 != nullptr, &fst);
    if (rc != MAC_OK) {
        c->rho = saved_rho;
        return st->status = rc;
    }
    MAC_CUDA_TRY(cudaMemcpyAsync(B.phiF, F.a64.phi, N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (phi_out) MAC_CUDA_TRY(cudaMemcpyAsync(phi_out, c->phin, N * sizeof(double), cudaMemcpyDeviceToDevice, s));

    AdjGeom G;
    for (int d = 0; d < 3; ++d) {
        G.n[d] = c->n[d];
        G.per[d] = (d < c->dm && c->bc_lo[d] == MAC_BC_PER) ? 1 : 0;
        G.idx[d] = 1.0 / c->dx[d];
    }
    G.dm = c->dm;
    G.va = c->va;
    G.p = beta0 ? (c->o.use_alt_energy_fix ? 2 : 1) : 0;
    G.d0 = F.d;
    const double* b0 = beta0 ? c->beta0 : nullptr;
    const double* b0e = beta0 ? c->beta0e : nullptr;

    // ---- adjoint right-hand side and solve with the same hierarchy
    k_adj_rhs<<<ceil_div((long)N, kB), kB, 0, s>>>(G, rho, b0, b0e, wx, wy, c->dm == 3 ? wz : wy,
                                                   c->scratch);
    MAC_CUDA_TRY(cudaGetLastError());
    rc = setup_rhs_from(c, c->scratch);
    if (rc) {
        c->rho = saved_rho;
        return st->status = rc;
    }
    MAC_CUDA_TRY(cudaMemsetAsync(F.a64.phi, 0, N * sizeof(double), s));
    const int solve_rc = run_solve(c, st);
    c->rho = saved_rho;
    if (solve_rc != MAC_OK && solve_rc != MAC_ERR_NOT_CONVERGED) return st->status = solve_rc;
    // nu = mu - mean(mu)
    k_partial_sum<<<nbp, kB, 0, s>>>((int)N, F.a64.phi, B.part);
    k_final_mean<<<1, 1024, 0, s>>>(nbp, (int)N, B.part, B.mean);
    MAC_CUDA_TRY(cudaGetLastError());

    // ---- per-face gradients
    for (int d = 0; d < c->dm; ++d) {
        const long nf = (long)(c->n[0] + (d == 0)) * (c->n[1] + (d == 1)) * (c->n[2] + (d == 2));
        FaceOut fo{dout[d], B.dh[d], B.db0[d]};
        k_adj_face<<<ceil_div(nf, kB), kB, 0, s>>>(G, d, rho, b0, b0e, uin[d], win[d], B.phiF,
                                                   F.a64.phi, B.mean, fo);
        MAC_CUDA_TRY(cudaGetLastError());
    }
    if (drinv) {
        k_adj_sigma<<<ceil_div((long)N, kB), kB, 0, s>>>(G, rho, B.dh[0], B.dh[1],
                                                         c->dm == 3 ? B.dh[2] : B.dh[1], drinv);
        MAC_CUDA_TRY(cudaGetLastError());
    }
    if (dmacrhs) {
        k_mu_to_nat<<<ceil_div((long)N, kB), kB, 0, s>>>(F.d, F.a64.phi, B.mean, dmacrhs);
        MAC_CUDA_TRY(cudaGetLastError());
    }
    if (dbeta0) {
        k_layer_sums<<<nr + 1, kB, 0, s>>>(G, B.db0[0], B.db0[1], c->dm == 3 ? B.db0[2] : B.db0[1],
                                           B.layer, B.layer + nr);
        MAC_CUDA_TRY(cudaGetLastError());
        std::vector<double> h(2 * nr + 1), cb(nr), g(nr);
        MAC_CUDA_TRY(cudaMemcpyAsync(h.data(), B.layer, (2 * nr + 1) * sizeof(double), cudaMemcpyDeviceToHost, s));
        MAC_CUDA_TRY(cudaMemcpyAsync(cb.data(), beta0, nr * sizeof(double), cudaMemcpyDeviceToHost, s));
        MAC_CUDA_TRY(cudaStreamSynchronize(s));
        for (int k = 0; k < nr; ++k) g[k] = h[k];
        cell_to_edge_vjp(nr, cb.data(), h.data() + nr, g.data());
        MAC_CUDA_TRY(cudaMemcpyAsync(dbeta0, g.data(), nr * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    MAC_CUDA_TRY(cudaStreamSynchronize(s));
    // the temporaries go back to the device now (the context keeps only its solver arrays)
    auto release = [&](void* p) {
        if (!p) return;
        for (size_t a = 0; a < c->allocations.size(); ++a)
            if (c->allocations[a] == p) {
                c->allocations.erase(c->allocations.begin() + (long)a);
                break;
            }
        cudaFree(p);
    };
    release(B.phiF);
    release(B.part);
    release(B.mean);
    release(B.layer);
    for (int d = 0; d < 3; ++d) {
        release(B.dh[d]);
        release(B.db0[d]);
    }
    st->vcycles += fst.vcycles;
    st->setup_ms += fst.setup_ms;
    st->solve_ms += fst.solve_ms;
    st->status = solve_rc;
    end_call_stats(c, st);
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return solve_rc;
}
