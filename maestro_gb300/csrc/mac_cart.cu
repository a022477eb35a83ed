// Spherical form of the MAC projection: beta0 given on every face (the 3-D face multifab
// beta0_cart_edge that MAESTRO's spherical geometry hands macproject instead of the planar 1-D
// arrays, Source/macproject.f90:103-109 checks, :155-161 U *= beta0, :194-201 solver beta *=
// beta0 (twice with the alternative energy fix), :236-241 U /= beta0).  The steps are the planar
// projection's with the per-layer factors replaced by face arrays:
//   beta_f = beta0_f^p 2 / (rho_lo + rho_hi)                       (mk_mac_coeffs, :698-738)
//   rh     = macrhs - div(beta0 U)                                   (divumac, :385-398)
//   solve  (-div beta grad) phi = rh                                 (mac_multigrid)
//   U      = (beta0 U - beta_f grad phi) / beta0 on every face       (mkumac, :908-975)
// The finest level's coefficients are stored (no per-layer tables to form them from rho), so
// the mixed-precision solve runs its finest FP32 level on stored FP32 coefficients like
// mac_multigrid.
#include <chrono>
#include <cstring>

#include "mac_internal.cuh"

namespace mac {
namespace {

struct CartParams {
    int n[3];
    int dm;
    int bc_lo[3], bc_hi[3];
    int p;          // beta0 power in the solver coefficient (1, or 2 with the energy fix)
    double idx[3];  // 1 / dx
};

__device__ __forceinline__ int face_index(const CartParams& P, int d, int i, int j, int k) {
    const int m0 = P.n[0] + (d == 0), m1 = P.n[1] + (d == 1);
    return i + m0 * (j + m1 * k);
}
__device__ __forceinline__ int cell_index(const CartParams& P, int i, int j, int k) {
    return i + P.n[0] * (j + P.n[1] * k);
}

// Solver beta on the faces normal to d.  Ghost density beyond a non-periodic boundary: the
// boundary cell's own value (first-order extrapolation), as the planar setup.  Each cell is
// checked for a positive, finite density once (as the high cell of its low face).
__global__ void k_cart_coef(CartParams P, int d, const double* __restrict__ rho,
                            const double* __restrict__ b0, double* __restrict__ beta,
                            int* __restrict__ err) {
    const int m[3] = {P.n[0] + (d == 0), P.n[1] + (d == 1), P.n[2] + (d == 2)};
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= m[0] || j >= m[1]) return;
    int hi[3] = {i, j, k}, lo[3] = {i, j, k};
    lo[d] -= 1;
    const bool own = hi[d] < P.n[d];
    if (hi[d] >= P.n[d]) hi[d] = P.bc_hi[d] == MAC_BC_PER ? 0 : P.n[d] - 1;
    if (lo[d] < 0) lo[d] = P.bc_lo[d] == MAC_BC_PER ? P.n[d] - 1 : 0;
    const double rh = rho[cell_index(P, hi[0], hi[1], hi[2])];
    const double rl = rho[cell_index(P, lo[0], lo[1], lo[2])];
    if (own && d == 0 && !positive_finite(rh)) atomicOr(err, 1);
    const int f = face_index(P, d, i, j, k);
    const double bb = b0[f];
    double v = 2.0 * recip_nr(rl + rh);
    v *= bb;
    if (P.p == 2) v *= bb;
    beta[f] = v;
}

// rh = macrhs - div(beta0 U), beta0 U formed face by face (natural cell layout out)
__global__ void k_cart_rhs(CartParams P, const double* __restrict__ ux,
                           const double* __restrict__ uy, const double* __restrict__ uz,
                           const double* __restrict__ bx, const double* __restrict__ by,
                           const double* __restrict__ bz, const double* __restrict__ macrhs,
                           double* __restrict__ rh) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= P.n[0] || j >= P.n[1]) return;
    const double* u[3] = {ux, uy, uz};
    const double* b[3] = {bx, by, bz};
    double dv = 0.0;
    for (int d = 0; d < P.dm; ++d) {
        const int fl = face_index(P, d, i, j, k);
        const int fh = face_index(P, d, i + (d == 0), j + (d == 1), k + (d == 2));
        dv += (u[d][fh] * b[d][fh] - u[d][fl] * b[d][fl]) * P.idx[d];
    }
    const int q = cell_index(P, i, j, k);
    rh[q] = macrhs ? macrhs[q] - dv : -dv;
}

// U = (beta0 U - beta_f grad phi) / beta0 on every face normal to d (phi natural layout);
// periodic faces wrap, Neumann faces keep their value, Dirichlet faces use the ghost
// -phi_boundary.
__global__ void k_cart_correct(CartParams P, int d, double* __restrict__ u,
                               const double* __restrict__ phi, const double* __restrict__ beta,
                               const double* __restrict__ b0) {
    const int m[3] = {P.n[0] + (d == 0), P.n[1] + (d == 1), P.n[2] + (d == 2)};
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= m[0] || j >= m[1]) return;
    const int f[3] = {i, j, k};
    const int q = f[d];
    int hi[3] = {i, j, k}, lo[3] = {i, j, k};
    lo[d] -= 1;
    double g;
    if (q > 0 && q < P.n[d]) {
        g = (phi[cell_index(P, hi[0], hi[1], hi[2])] - phi[cell_index(P, lo[0], lo[1], lo[2])]) *
            P.idx[d];
    } else if ((q == 0 && P.bc_lo[d] == MAC_BC_PER) || (q == P.n[d] && P.bc_hi[d] == MAC_BC_PER)) {
        hi[d] = 0;
        lo[d] = P.n[d] - 1;
        g = (phi[cell_index(P, hi[0], hi[1], hi[2])] - phi[cell_index(P, lo[0], lo[1], lo[2])]) *
            P.idx[d];
    } else if (q == 0) {
        g = P.bc_lo[d] == MAC_BC_DIR ? 2.0 * phi[cell_index(P, hi[0], hi[1], hi[2])] * P.idx[d]
                                      : 0.0;
    } else {
        g = P.bc_hi[d] == MAC_BC_DIR ? -2.0 * phi[cell_index(P, lo[0], lo[1], lo[2])] * P.idx[d]
                                      : 0.0;
    }
    const int fi = face_index(P, d, i, j, k);
    const double bb = b0[fi];
    double x = u[fi] * bb;
    x = fma(-beta[fi], g, x);
    u[fi] = x / bb;
}

CartParams cart_params(const mac_ctx* c) {
    CartParams P;
    for (int d = 0; d < 3; ++d) {
        P.n[d] = c->n[d];
        P.bc_lo[d] = c->bc_lo[d];
        P.bc_hi[d] = c->bc_hi[d];
        P.idx[d] = 1.0 / c->dx[d];
    }
    P.dm = c->dm;
    P.p = c->o.use_alt_energy_fix ? 2 : 1;
    return P;
}

Grid3 face_grid(const mac_ctx* c, int d) {
    return grid3(c->n[0] + (d == 0), c->n[1] + (d == 1), c->n[2] + (d == 2));
}

size_t face_count(const mac_ctx* c, int d) {
    return (size_t)(c->n[0] + (d == 0)) * (c->n[1] + (d == 1)) * (c->n[2] + (d == 2));
}

int ensure_cart(mac_ctx* c, bool with_b0) {
    for (int d = 0; d < c->dm; ++d) {
        if (!c->cbeta[d]) {
            void* p = nullptr;
            if (alloc_device(c, &p, sizeof(double) * face_count(c, d))) return MAC_ERR_ALLOC;
            c->cbeta[d] = static_cast<double*>(p);
        }
        if (with_b0 && !c->cb0[d]) {
            void* p = nullptr;
            if (alloc_device(c, &p, sizeof(double) * face_count(c, d))) return MAC_ERR_ALLOC;
            c->cb0[d] = static_cast<double*>(p);
        }
    }
    return MAC_OK;
}

// The projection on whole-domain device arrays in c->u / c->rho / c->phin with beta0 faces b0.
int core_cart(mac_ctx* c, const double* macrhs, const double* const* b0, mac_stats* st) {
    Level& F = c->lev[0];
    cudaEventRecord(c->ev[0], c->stream);
    int rc = set_call_state(c, false);
    if (rc) return rc;
    set_otf_mode(c, false);
    rc = ensure_cart(c, false);
    if (rc) return rc;
    const CartParams P = cart_params(c);
    MAC_CUDA_TRY(cudaMemsetAsync(c->red.counters, 0, 4 * sizeof(int), c->stream));
    for (int d = 0; d < c->dm; ++d) {
        const Grid3 g = face_grid(c, d);
        k_cart_coef<<<g.grid, g.block, 0, c->stream>>>(P, d, c->rho, b0[d], c->cbeta[d],
                                                       c->red.counters + 1);
        MAC_CUDA_TRY(cudaGetLastError());
        ++c->issued;
    }
    rc = setup_fine_from_faces(c, c->cbeta[0], c->cbeta[1], c->dm == 3 ? c->cbeta[2] : nullptr,
                               nullptr, false);
    if (rc) return rc;
    rc = setup_coarse_levels(c);
    if (rc) return rc;
    {
        const Grid3 g = grid3(c->n[0], c->n[1], c->n[2]);
        k_cart_rhs<<<g.grid, g.block, 0, c->stream>>>(P, c->u[0], c->u[1], c->u[2], b0[0], b0[1],
                                                      c->dm == 3 ? b0[2] : nullptr, macrhs,
                                                      c->scratch);
        MAC_CUDA_TRY(cudaGetLastError());
        ++c->issued;
    }
    rc = setup_rhs_from(c, c->scratch, c->phin);   // also moves phi into the level-0 layout
    if (rc) return rc;
    cudaEventRecord(c->ev[1], c->stream);
    const long long setup_kernels = c->issued;
    const int solve_rc = run_solve(c, st);
    if (solve_rc != MAC_OK && solve_rc != MAC_ERR_NOT_CONVERGED) return solve_rc;
    cudaEventRecord(c->ev[2], c->stream);
    const long long before_corr = c->issued;
    rc = level0_to_natural(c, F.a64.phi, c->phin);
    if (rc) return rc;
    for (int d = 0; d < c->dm; ++d) {
        const Grid3 g = face_grid(c, d);
        k_cart_correct<<<g.grid, g.block, 0, c->stream>>>(P, d, c->u[d], c->phin, c->cbeta[d],
                                                          b0[d]);
        MAC_CUDA_TRY(cudaGetLastError());
        ++c->issued;
    }
    c->ktime_launches[MAC_KT_CORRECT] += (int)(c->issued - before_corr);
    c->ktime_launches[MAC_KT_SETUP] += (int)setup_kernels;
    cudaEventRecord(c->ev[3], c->stream);
    MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    float a = 0.f, b = 0.f, cc = 0.f;
    cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
    cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
    cudaEventElapsedTime(&cc, c->ev[2], c->ev[3]);
    st->setup_ms = a + cc;
    st->solve_ms = b;
    c->ktime_ms[MAC_KT_SETUP] += a;
    c->ktime_ms[MAC_KT_CORRECT] += cc;
    return solve_rc;
}

}  // namespace
}  // namespace mac

using namespace mac;

extern "C" {

int mac_macproject_cart_dense(mac_ctx* c, double* ux, double* uy, double* uz, double* phi,
                              const double* rho, const double* macrhs, const double* b0x,
                              const double* b0y, const double* b0z, mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if (!c || !ux || !uy || (c->dm == 3 && !uz) || !phi || !rho || !b0x || !b0y ||
        (c->dm == 3 && !b0z))
        return st->status = MAC_ERR_INVALID;
    const auto t0 = std::chrono::steady_clock::now();
    begin_call_stats(c, st);
    double* saved_u[3] = {c->u[0], c->u[1], c->u[2]};
    double* saved_rho = c->rho;
    double* saved_phin = c->phin;
    c->u[0] = ux;
    c->u[1] = uy;
    c->u[2] = c->dm == 3 ? uz : nullptr;
    c->rho = const_cast<double*>(rho);
    c->phin = phi;
    const double* b0[3] = {b0x, b0y, c->dm == 3 ? b0z : nullptr};
    const int rc = core_cart(c, macrhs, b0, st);
    c->u[0] = saved_u[0];
    c->u[1] = saved_u[1];
    c->u[2] = saved_u[2];
    c->rho = saved_rho;
    c->phin = saved_phin;
    st->status = rc;
    st->total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    end_call_stats(c, st);
    report_call(c, "macproject_cart_dense", st);
    return rc;
}

int mac_macproject_cart(mac_ctx* c, int ptr_kind, double* const* umac, int ng_u,
                        double* const* phi, int ng_phi, const double* const* rho, int ng_rho,
                        int rho_ncomp, int rho_comp, const double* const* macrhs, int ng_rhs,
                        const double* const* beta0_cart_edge, int ng_b, mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if (!c || !umac || !phi || !rho || !beta0_cart_edge) return st->status = MAC_ERR_INVALID;
    if (ptr_kind != MAC_PTR_HOST && ptr_kind != MAC_PTR_DEVICE) return st->status = MAC_ERR_INVALID;
    if (ng_u < 0 || ng_phi < 0 || ng_rho < 0 || ng_rhs < 0 || ng_b < 0 || rho_ncomp < 1 ||
        rho_comp < 0 || rho_comp >= rho_ncomp)
        return st->status = MAC_ERR_INVALID;
    const int nb = c->g.nboxes;
    for (int b = 0; b < nb; ++b) {
        if (!phi[b] || !rho[b] || (macrhs && !macrhs[b])) return st->status = MAC_ERR_INVALID;
        for (int d = 0; d < c->dm; ++d)
            if (!umac[d * nb + b] || !beta0_cart_edge[d * nb + b])
                return st->status = MAC_ERR_INVALID;
    }
    const auto t0 = std::chrono::steady_clock::now();
    begin_call_stats(c, st);
    int rc = ensure_cart(c, true);
    if (!rc && ptr_kind == MAC_PTR_HOST) {
        size_t need = host_fab_elems(c, -1, ng_rho) + host_fab_elems(c, -1, ng_phi);
        for (int d = 0; d < c->dm; ++d)
            need += host_fab_elems(c, d, ng_u) + host_fab_elems(c, d, ng_b);
        if (macrhs) need += host_fab_elems(c, -1, ng_rhs);
        rc = staging_reserve(c, need);
    }
    for (int d = 0; d < c->dm && !rc; ++d)
        rc = gather_faces(c, ptr_kind, beta0_cart_edge + d * nb, ng_b, d, c->cb0[d]);
    if (!rc) rc = gather_cells(c, ptr_kind, rho, ng_rho, rho_ncomp, rho_comp, c->rho);
    for (int d = 0; d < c->dm && !rc; ++d)
        rc = gather_faces(c, ptr_kind, (const double* const*)(umac + d * nb), ng_u, d, c->u[d]);
    if (!rc && macrhs) rc = gather_cells(c, ptr_kind, macrhs, ng_rhs, 1, 0, c->rhs);
    if (!rc) rc = gather_cells(c, ptr_kind, (const double* const*)phi, ng_phi, 1, 0, c->phin);
    int solve_rc = MAC_OK;
    if (!rc) {
        const double* b0[3] = {c->cb0[0], c->cb0[1], c->cb0[2]};
        solve_rc = core_cart(c, macrhs ? c->rhs : nullptr, b0, st);
        if (solve_rc != MAC_OK && solve_rc != MAC_ERR_NOT_CONVERGED) rc = solve_rc;
    }
    for (int d = 0; d < c->dm && !rc; ++d)
        rc = scatter_faces(c, ptr_kind, umac + d * nb, ng_u, d, c->u[d]);
    if (!rc) rc = scatter_cells(c, ptr_kind, phi, ng_phi, c->phin);
    cudaError_t e = cudaStreamSynchronize(c->xfer);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess && !rc) {
        set_last_cuda_error(e, "cudaStreamSynchronize", __FILE__, __LINE__);
        rc = MAC_ERR_CUDA;
    }
    if (!rc) rc = solve_rc;
    st->status = rc;
    st->total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    end_call_stats(c, st);
    report_call(c, "macproject_cart", st);
    return rc;
}

}  // extern "C"
