// Producers of the MAC projection's inputs, on the device, so that the predictor and corrector MAC
// steps can stay on the GPU:
//   make_macrhs      (Source/make_macrhs.f90:28-107 driver, :135-178 2-D, :184-240 3-D planar):
//     macrhs = beta0(r) (S_cc - Sbar(r) + delta_gamma1_term)
//     and, when dpdt_factor > 0: delta_chi = 0 first on a predictor call; on cells below the
//     base cutoff (r < base_cutoff_density_coord) delta_chi += dpdt_factor delta_p_term /
//     (dt gamma1bar(r) p0(r)) and macrhs += beta0(r) delta_chi
//   make_at_halftime (Source/make_at_halftime.f90:82-190): half = (old + new) / 2
// r is the vertical index (y in 2-D, z in 3-D).  Planar geometry only (the spherical form is a
// separate path).
#include <chrono>
#include <cstring>
#include <vector>

#include "mac_internal.cuh"

namespace mac {
namespace {

constexpr int kB = 256;

struct MacrhsParams {
    int n[3];
    int va;                 // vertical direction (index of r)
    int have_chi;           // dpdt_factor > 0
    int predictor;          // zero delta_chi first
    int cutoff;             // base_cutoff_density_coord
    double dpdt_factor, dt;
};

__global__ void __launch_bounds__(kB)
k_make_macrhs(MacrhsParams P, double* __restrict__ rhs, const double* __restrict__ S,
              const double* __restrict__ dg1, const double* __restrict__ Sbar,
              const double* __restrict__ beta0, const double* __restrict__ gamma1bar,
              const double* __restrict__ p0, const double* __restrict__ dp,
              double* __restrict__ chi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= P.n[0] || j >= P.n[1]) return;
    const long q = i + (long)P.n[0] * (j + (long)P.n[1] * k);
    const int r = P.va == 2 ? k : j;
    const double b0 = beta0[r];
    double v = b0 * (S[q] - Sbar[r] + dg1[q]);
    if (P.have_chi) {
        double c = P.predictor ? 0.0 : chi[q];
        if (r < P.cutoff) {
            c = c + P.dpdt_factor * dp[q] / (P.dt * gamma1bar[r] * p0[r]);
            v = v + b0 * c;
        }
        chi[q] = c;
    }
    rhs[q] = v;
}

__global__ void __launch_bounds__(kB)
k_halftime(long n, double* __restrict__ half, const double* __restrict__ a,
           const double* __restrict__ b) {
    const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q < n) half[q] = 0.5 * (a[q] + b[q]);
}

int run_make_macrhs(mac_ctx* c, double* rhs, const double* S, const double* dg1, const double* Sbar,
                    const double* beta0, const double* gamma1bar, const double* p0,
                    const double* dp, double* chi, double dt, double dpdt_factor, int cutoff,
                    int is_predictor) {
    MacrhsParams P;
    for (int d = 0; d < 3; ++d) P.n[d] = c->n[d];
    P.va = c->va;
    P.have_chi = dpdt_factor > 0.0 ? 1 : 0;
    P.predictor = is_predictor ? 1 : 0;
    P.cutoff = cutoff;
    P.dpdt_factor = dpdt_factor;
    P.dt = dt;
    const Grid3 g = grid3(c->n[0], c->n[1], c->n[2]);
    k_make_macrhs<<<g.grid, g.block, 0, c->stream>>>(P, rhs, S, dg1, Sbar, beta0, gamma1bar, p0,
                                                     dp, chi);
    MAC_CUDA_TRY(cudaGetLastError());
    return MAC_OK;
}

// The 1-D base-state arrays (nr entries) in device memory: copied into ctx storage from the
// host, or used in place when already on the device.
struct Base1d {
    const double* p[4];
};
int base_arrays(mac_ctx* c, int ptr_kind, const double* const* in, double* store, Base1d* out) {
    const int nr = c->n[c->va];
    for (int a = 0; a < 4; ++a) {
        if (ptr_kind == MAC_PTR_DEVICE) {
            out->p[a] = in[a];
        } else {
            MAC_CUDA_TRY(cudaMemcpyAsync(store + (size_t)a * nr, in[a], sizeof(double) * nr,
                                         cudaMemcpyHostToDevice, c->stream));
            out->p[a] = store + (size_t)a * nr;
        }
    }
    return MAC_OK;
}

}  // namespace
}  // namespace mac

using namespace mac;

extern "C" {

int mac_make_macrhs_dense(mac_ctx* c, double* macrhs, const double* S_cc,
                          const double* delta_gamma1_term, const double* Sbar,
                          const double* beta0, const double* gamma1bar, const double* p0,
                          const double* delta_p_term, double* delta_chi, double dt,
                          double dpdt_factor, int base_cutoff_density_coord, int is_predictor) {
    if (!c || !macrhs || !S_cc || !delta_gamma1_term || !Sbar || !beta0) return MAC_ERR_INVALID;
    if (dpdt_factor > 0.0 && (!gamma1bar || !p0 || !delta_p_term || !delta_chi || !(dt > 0.0)))
        return MAC_ERR_INVALID;
    int rc = run_make_macrhs(c, macrhs, S_cc, delta_gamma1_term, Sbar, beta0, gamma1bar, p0,
                             delta_p_term, delta_chi, dt, dpdt_factor, base_cutoff_density_coord,
                             is_predictor);
    if (rc) return rc;
    MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MAC_OK;
}

int mac_make_macrhs(mac_ctx* c, int ptr_kind, double* const* macrhs, int ng_rh,
                    const double* const* S_cc, int ng_sr, const double* const* delta_gamma1_term,
                    int ng_dg, const double* Sbar, const double* beta0, const double* gamma1bar,
                    const double* p0, const double* const* delta_p_term, int ng_dp,
                    double* const* delta_chi, int ng_d, double dt, double dpdt_factor,
                    int base_cutoff_density_coord, int is_predictor) {
    if (!c || !macrhs || !S_cc || !delta_gamma1_term || !Sbar || !beta0) return MAC_ERR_INVALID;
    if (ptr_kind != MAC_PTR_HOST && ptr_kind != MAC_PTR_DEVICE) return MAC_ERR_INVALID;
    if (ng_rh < 0 || ng_sr < 0 || ng_dg < 0 || ng_dp < 0 || ng_d < 0) return MAC_ERR_INVALID;
    const bool chi = dpdt_factor > 0.0;
    if (chi && (!gamma1bar || !p0 || !delta_p_term || !delta_chi || !(dt > 0.0)))
        return MAC_ERR_INVALID;
    const int nb = c->g.nboxes;
    for (int b = 0; b < nb; ++b) {
        if (!macrhs[b] || !S_cc[b] || !delta_gamma1_term[b]) return MAC_ERR_INVALID;
        if (chi && (!delta_p_term[b] || !delta_chi[b])) return MAC_ERR_INVALID;
    }
    // whole-domain scratch: S -> u[0], dg1 -> u[1], delta_p -> scratch, delta_chi -> phin,
    // macrhs -> rhs; host base-state arrays -> base1d
    int rc = MAC_OK;
    if (ptr_kind == MAC_PTR_HOST) {
        size_t need = 2 * host_fab_elems(c, -1, ng_sr) + host_fab_elems(c, -1, ng_rh);
        if (chi) need += host_fab_elems(c, -1, ng_dp) + 2 * host_fab_elems(c, -1, ng_d);
        rc = staging_reserve(c, need);
    }
    const double* in1d[4] = {Sbar, beta0, chi ? gamma1bar : Sbar, chi ? p0 : Sbar};
    Base1d B;
    if (!rc) rc = base_arrays(c, ptr_kind, in1d, c->base1d, &B);
    if (!rc) rc = gather_cells(c, ptr_kind, S_cc, ng_sr, 1, 0, c->u[0]);
    if (!rc) rc = gather_cells(c, ptr_kind, delta_gamma1_term, ng_dg, 1, 0, c->u[1]);
    if (!rc && chi) rc = gather_cells(c, ptr_kind, delta_p_term, ng_dp, 1, 0, c->scratch);
    if (!rc && chi && !is_predictor)
        rc = gather_cells(c, ptr_kind, (const double* const*)delta_chi, ng_d, 1, 0, c->phin);
    if (!rc)
        rc = run_make_macrhs(c, c->rhs, c->u[0], c->u[1], B.p[0], B.p[1], B.p[2], B.p[3],
                             c->scratch, c->phin, dt, dpdt_factor, base_cutoff_density_coord,
                             is_predictor);
    if (!rc) rc = scatter_cells(c, ptr_kind, macrhs, ng_rh, c->rhs);
    if (!rc && chi) rc = scatter_cells(c, ptr_kind, delta_chi, ng_d, c->phin);
    cudaError_t e = cudaStreamSynchronize(c->xfer);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess && !rc) {
        set_last_cuda_error(e, "cudaStreamSynchronize", __FILE__, __LINE__);
        rc = MAC_ERR_CUDA;
    }
    return rc;
}

int mac_make_at_halftime(mac_ctx* c, int ptr_kind, double* const* half, int ng_half, int out_comp,
                         int half_ncomp, const double* const* sold, int ng_old,
                         const double* const* snew, int ng_new, int in_comp, int s_ncomp) {
    if (!c || !half || !sold || !snew) return MAC_ERR_INVALID;
    if (ptr_kind != MAC_PTR_HOST && ptr_kind != MAC_PTR_DEVICE) return MAC_ERR_INVALID;
    if (ng_half < 0 || ng_old < 0 || ng_new < 0 || out_comp < 0 || out_comp >= half_ncomp ||
        in_comp < 0 || in_comp >= s_ncomp)
        return MAC_ERR_INVALID;
    if (half_ncomp != 1) return MAC_ERR_UNSUPPORTED;   // one-component output fabs
    const int nb = c->g.nboxes;
    for (int b = 0; b < nb; ++b)
        if (!half[b] || !sold[b] || !snew[b]) return MAC_ERR_INVALID;
    int rc = MAC_OK;
    if (ptr_kind == MAC_PTR_HOST)
        rc = staging_reserve(c, host_fab_elems(c, -1, ng_old) + host_fab_elems(c, -1, ng_new) +
                                    host_fab_elems(c, -1, ng_half));
    if (!rc) rc = gather_cells(c, ptr_kind, sold, ng_old, s_ncomp, in_comp, c->u[0]);
    if (!rc) rc = gather_cells(c, ptr_kind, snew, ng_new, s_ncomp, in_comp, c->u[1]);
    const long n = (long)c->n[0] * c->n[1] * c->n[2];
    if (!rc) {
        k_halftime<<<(unsigned)((n + kB - 1) / kB), kB, 0, c->stream>>>(n, c->scratch, c->u[0],
                                                                        c->u[1]);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_last_cuda_error(e, "k_halftime", __FILE__, __LINE__);
            rc = MAC_ERR_CUDA;
        }
    }
    if (!rc) rc = scatter_cells(c, ptr_kind, half, ng_half, c->scratch);
    cudaError_t e = cudaStreamSynchronize(c->xfer);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess && !rc) {
        set_last_cuda_error(e, "cudaStreamSynchronize", __FILE__, __LINE__);
        rc = MAC_ERR_CUDA;
    }
    return rc;
}

}  // extern "C"
