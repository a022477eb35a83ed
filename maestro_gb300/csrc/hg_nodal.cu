// Nodal (HG) projection on the GPU: the node / cell functions of hg_nodal.cuh as kernels, the
// executor of hg::project on device arrays, and the C ABI entry mac_hgproject_dense.
//
// One thread per node or cell, FP64, natural layout; the nodal hierarchy (coarse sigma and the
// node arrays of every multigrid level) lives in the context and is allocated on first use.  All
// launches go to the context's stream; the host reads one residual norm per V-cycle.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "hg_nodal.cuh"
#include "mac_internal.cuh"

namespace mac {

namespace {

constexpr int kThreads = 256;
constexpr int kReduceBlocks = 1024;

#define HG_LOOP(N) for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < (N); \
                        idx += (long)gridDim.x * blockDim.x)

__global__ void k_hg_defect(hg::Geo G, hg::Lev L, const double* phi, const double* f, double* r,
                            long N) {
    HG_LOOP(N) hg::defect_node(G, L, idx, phi, f, r);
}
__global__ void k_hg_gs(hg::Geo G, hg::Lev L, int colour, double* phi, const double* f, long N) {
    HG_LOOP(N) hg::gs_node(G, L, idx, colour, phi, f);
}
__global__ void k_hg_restrict(hg::Geo G, hg::Lev F, hg::Lev K, const double* rF, double* fK,
                              long N) {
    HG_LOOP(N) hg::restrict_node(G, F, K, idx, rF, fK);
}
__global__ void k_hg_prolong(hg::Geo G, hg::Lev K, hg::Lev F, const double* eK, double* phiF,
                             long N) {
    HG_LOOP(N) hg::prolong_node(G, K, F, idx, eK, phiF);
}
__global__ void k_hg_coarsen(hg::Geo G, hg::Lev F, hg::Lev K, double* sK, long N) {
    HG_LOOP(N) hg::coarsen_sig_cell(G, F, K, idx, sK);
}
__global__ void k_hg_finish(hg::Geo G, hg::Lev L, double* x, long N) {
    HG_LOOP(N) hg::finish_node(G, L, idx, x);
}
__global__ void k_hg_uvec(hg::Geo G, long nc, int proj_type, double dt, double* unew,
                          const double* uold, const double* gpi, const double* rhohalf,
                          const double* b0, int alt, double* sig) {
    HG_LOOP(nc) hg::uvec_cell(G, idx, nc, proj_type, dt, unew, uold, gpi, rhohalf, b0, alt, sig);
}
__global__ void k_hg_divu(hg::Geo G, hg::Lev L, const double* u, const double* b0,
                          const double* nodalrhs, double* rh, long N) {
    HG_LOOP(N) hg::divu_node(G, L, idx, u, b0, nodalrhs, rh);
}
__global__ void k_hg_update(hg::Geo G, hg::Lev L, int proj_type, double dt, const double* phi,
                            double* unew, const double* uold, double* gpi, const double* rhohalf,
                            const double* b0, int alt, long N) {
    HG_LOOP(N) hg::update_cell(G, L, idx, proj_type, dt, phi, unew, uold, gpi, rhohalf, b0, alt);
}
__global__ void k_hg_update_pi(hg::Lev L, int proj_type, double dt, const double* phi, double* pi,
                               long N) {
    HG_LOOP(N) hg::update_pi_node(L, idx, proj_type, dt, phi, pi);
}

// nu colour-ordered Gauss-Seidel sweeps of the coarsest level in one block.  An odd periodic
// extent couples nodes of one colour across the wrap: then one thread sweeps in order.
__global__ void k_hg_bottom(hg::Geo G, hg::Lev L, double* phi, const double* f, int nu, long N) {
    bool serial = false;
    for (int d = 0; d < G.dm; ++d) serial = serial || (G.per[d] && (L.n[d] & 1));
    const long start = serial ? 0 : threadIdx.x;
    const long step = serial ? 1 : blockDim.x;
    const bool active = !serial || threadIdx.x == 0;
    for (int s = 0; s < nu; ++s)
        for (int colour = 0; colour < (1 << G.dm); ++colour) {
            if (active)
                for (long idx = start; idx < N; idx += step) hg::gs_node(G, L, idx, colour, phi, f);
            __syncthreads();
        }
}

// Per-block partials over the unknown nodes: [0] sum, [1] max |x|, [2] NaN count, [3] count.
__global__ void k_hg_reduce(hg::Geo G, hg::Lev L, const double* x, double* part, long N) {
    __shared__ double s[4][kThreads / 32];
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    HG_LOOP(N) {
        int p[3];
        hg::node_coords(L, idx, p);
        if (!hg::is_unknown(G, L, p)) continue;
        const double v = x[idx];
        if (v != v) {
            a[2] += 1.0;
            continue;
        }
        a[0] += v;
        a[1] = fmax(a[1], fabs(v));
        a[3] += 1.0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        a[0] += __shfl_down_sync(0xffffffffu, a[0], o);
        a[1] = fmax(a[1], __shfl_down_sync(0xffffffffu, a[1], o));
        a[2] += __shfl_down_sync(0xffffffffu, a[2], o);
        a[3] += __shfl_down_sync(0xffffffffu, a[3], o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 4; ++k) s[k][w] = a[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < kThreads / 32; ++q) {
            a[0] += s[0][q];
            a[1] = fmax(a[1], s[1][q]);
            a[2] += s[2][q];
            a[3] += s[3][q];
        }
        for (int k = 0; k < 4; ++k) part[4 * blockIdx.x + k] = a[k];
    }
}

// out[0] sum, [1] max, [2] NaN count, [3] count, [4] mean; one block, fixed order.
__global__ void k_hg_reduce_finish(const double* part, int nparts, double* out) {
    __shared__ double s[4][kThreads];
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    for (int q = threadIdx.x; q < nparts; q += blockDim.x) {
        a[0] += part[4 * q];
        a[1] = fmax(a[1], part[4 * q + 1]);
        a[2] += part[4 * q + 2];
        a[3] += part[4 * q + 3];
    }
    for (int k = 0; k < 4; ++k) s[k][threadIdx.x] = a[k];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s[0][threadIdx.x] += s[0][threadIdx.x + w];
            s[1][threadIdx.x] = fmax(s[1][threadIdx.x], s[1][threadIdx.x + w]);
            s[2][threadIdx.x] += s[2][threadIdx.x + w];
            s[3][threadIdx.x] += s[3][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < 4; ++k) out[k] = s[k][0];
        out[4] = s[3][0] > 0.0 ? s[0][0] / s[3][0] : 0.0;
    }
}

__global__ void k_hg_sub_mean(hg::Geo G, hg::Lev L, double* x, const double* m, long N) {
    const double v = *m;
    HG_LOOP(N) {
        int p[3];
        hg::node_coords(L, idx, p);
        if (hg::is_unknown(G, L, p)) x[idx] -= v;
    }
}

// A rhohalf that is not positive and finite, or a beta0 that is not, raises flag[0].
__global__ void k_hg_check(const double* rhohalf, const double* b0, int* flag, long N) {
    HG_LOOP(N) {
        const double r = rhohalf[idx];
        const double b = b0 ? b0[idx] : 1.0;
        if (!(r > 0.0) || !(r < INFINITY) || !(b > 0.0) || !(b < INFINITY)) atomicExch(flag, 1);
    }
}

inline int blocks_for(long n, int sms) {
    const long b = (n + kThreads - 1) / kThreads;
    const long cap = (long)std::max(1, sms) * 16;
    return (int)std::max(1L, std::min(b, cap));
}

}  // namespace

struct HgState {
    hg::Geo geo{};
    int dense = -1;
    struct Level {
        hg::Lev lev{};
        double* sig = nullptr;
        double* buf[hg::kNumBufs] = {};
        long nn = 0, nc = 0;
    };
    std::vector<Level> L;
    double* part = nullptr;
    double* out = nullptr;
    double* h_out = nullptr;
    int* flag = nullptr;
    int* h_flag = nullptr;
    std::vector<void*> allocs;
};

void hg_release(mac_ctx* c) {
    HgState* H = c->hgs;
    if (!H) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (void* p : H->allocs) cudaFree(p);
    if (H->h_out) cudaFreeHost(H->h_out);
    if (H->h_flag) cudaFreeHost(H->h_flag);
    delete H;
    c->hgs = nullptr;
}

namespace {

template <typename T>
int hg_alloc(HgState* H, T** p, size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return MAC_ERR_ALLOC;
    }
    H->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return MAC_OK;
}

// The nodal hierarchy of the context's geometry: level 0 at the context's cells, coarsened by 2
// while every active extent is even and at least 4.
int hg_ensure(mac_ctx* c) {
    if (c->hgs) return MAC_OK;
    HgState* H = new HgState();
    c->hgs = H;
    hg::Geo& G = H->geo;
    G.dm = c->dm;
    for (int d = 0; d < 3; ++d) {
        G.per[d] = d < c->dm && c->bc_lo[d] == MAC_BC_PER;
        G.dlo[d] = d < c->dm && c->bc_lo[d] == MAC_BC_DIR;
        G.dhi[d] = d < c->dm && c->bc_hi[d] == MAC_BC_DIR;
    }
    int n[3], rc = MAC_OK;
    double h[3];
    for (int d = 0; d < 3; ++d) {
        n[d] = d < c->dm ? c->n[d] : 1;
        h[d] = c->dx[d];
    }
    while (true) {
        HgState::Level S;
        for (int d = 0; d < 3; ++d) {
            S.lev.n[d] = n[d];
            S.lev.nn[d] = d < c->dm ? n[d] + 1 : 1;
            S.lev.h[d] = h[d];
        }
        S.nn = hg::nnodes(S.lev);
        S.nc = hg::ncells(S.lev);
        rc = hg_alloc(H, &S.sig, (size_t)S.nc);
        for (int b = 0; b < hg::kNumBufs && !rc; ++b) rc = hg_alloc(H, &S.buf[b], (size_t)S.nn);
        if (rc) break;
        S.lev.sig = S.sig;
        H->L.push_back(S);
        bool more = (int)H->L.size() < hg::kMaxLevels;
        for (int d = 0; d < c->dm; ++d) more = more && n[d] % 2 == 0 && n[d] >= 4;
        if (!more) break;
        for (int d = 0; d < c->dm; ++d) {
            n[d] /= 2;
            h[d] *= 2;
        }
    }
    if (!rc) rc = hg_alloc(H, &H->part, (size_t)4 * kReduceBlocks);
    if (!rc) rc = hg_alloc(H, &H->out, 8);
    if (!rc) rc = hg_alloc(H, &H->flag, 1);
    if (!rc && (cudaMallocHost((void**)&H->h_out, 8 * sizeof(double)) != cudaSuccess ||
                cudaMallocHost((void**)&H->h_flag, sizeof(int)) != cudaSuccess)) {
        cudaGetLastError();
        rc = MAC_ERR_ALLOC;
    }
    if (rc) hg_release(c);
    return rc;
}

struct HgExec {
    mac_ctx* c;
    HgState* H;
    int nlev;
    hg::Geo geo;
    bool singular;
    int err = MAC_OK;
    // this call
    int proj_type = hg::kRegular;
    double dt = 1.0;
    double* unew = nullptr;
    const double* uold = nullptr;
    double* gpi = nullptr;
    const double* rhohalf = nullptr;
    double* pi = nullptr;
    const double* b0 = nullptr;
    const double* nodalrhs = nullptr;
    int alt = 0;

    hg::Lev lev(int l) const { return H->L[l].lev; }
    double* buf(int l, int w) const { return H->L[l].buf[w]; }
    long nn(int l) const { return H->L[l].nn; }
    long nc(int l) const { return H->L[l].nc; }
    int blocks(long n) const { return blocks_for(n, c->sms); }
    int error() const { return err; }
    void launched() {
        ++c->issued;
        if (!err && cudaPeekAtLastError() != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "hg kernel launch", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
        }
    }

    void defect(int l, const double* phi, const double* f, double* r) {
        k_hg_defect<<<blocks(nn(l)), kThreads, 0, c->stream>>>(geo, lev(l), phi, f, r, nn(l));
        launched();
    }
    void gs(int l, double* phi, const double* f, int nu) {
        for (int s = 0; s < nu; ++s)
            for (int colour = 0; colour < (1 << geo.dm); ++colour) {
                k_hg_gs<<<blocks(nn(l)), kThreads, 0, c->stream>>>(geo, lev(l), colour, phi, f, nn(l));
                launched();
            }
    }
    void bottom_gs(int l, double* phi, const double* f, int nu) {
        k_hg_bottom<<<1, 1024, 0, c->stream>>>(geo, lev(l), phi, f, nu, nn(l));
        launched();
    }
    void restrict_to(int lc, const double* rF, double* fK) {
        k_hg_restrict<<<blocks(nn(lc)), kThreads, 0, c->stream>>>(geo, lev(lc - 1), lev(lc), rF, fK, nn(lc));
        launched();
    }
    void prolong(int lc, const double* eK, double* phiF) {
        k_hg_prolong<<<blocks(nn(lc - 1)), kThreads, 0, c->stream>>>(geo, lev(lc), lev(lc - 1), eK, phiF, nn(lc - 1));
        launched();
    }
    void zero(int l, double* x) {
        if (!err && cudaMemsetAsync(x, 0, sizeof(double) * nn(l), c->stream) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "cudaMemsetAsync", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
        }
    }
    void finish(int l, double* x) {
        k_hg_finish<<<blocks(nn(l)), kThreads, 0, c->stream>>>(geo, lev(l), x, nn(l));
        launched();
    }
    void reduce(int l, const double* x) {
        const int nb = std::min(kReduceBlocks, blocks(nn(l)));
        k_hg_reduce<<<nb, kThreads, 0, c->stream>>>(geo, lev(l), x, H->part, nn(l));
        launched();
        k_hg_reduce_finish<<<1, kThreads, 0, c->stream>>>(H->part, nb, H->out);
        launched();
    }
    double unknown_max(int l, const double* x) {
        reduce(l, x);
        if (err) return NAN;
        if (cudaMemcpyAsync(H->h_out, H->out, 5 * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
            cudaStreamSynchronize(c->stream) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "hg reduction", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
            return NAN;
        }
        return H->h_out[2] > 0.0 ? NAN : H->h_out[1];
    }
    void sub_unknown_mean(int l, double* x) {
        reduce(l, x);
        k_hg_sub_mean<<<blocks(nn(l)), kThreads, 0, c->stream>>>(geo, lev(l), x, H->out + 4, nn(l));
        launched();
    }

    void uvec() {
        k_hg_uvec<<<blocks(nc(0)), kThreads, 0, c->stream>>>(geo, nc(0), proj_type, dt, unew, uold, gpi,
                                                            rhohalf, b0, alt, H->L[0].sig);
        launched();
    }
    int build_levels() {
        for (size_t l = 1; l < H->L.size(); ++l) {
            k_hg_coarsen<<<blocks(nc((int)l)), kThreads, 0, c->stream>>>(geo, lev((int)l - 1), lev((int)l),
                                                                       H->L[l].sig, nc((int)l));
            launched();
        }
        return err;
    }
    void divu() {
        k_hg_divu<<<blocks(nn(0)), kThreads, 0, c->stream>>>(geo, lev(0), unew, b0, nodalrhs,
                                                            buf(0, hg::kF), nn(0));
        launched();
    }
    void update() {
        k_hg_update<<<blocks(nc(0)), kThreads, 0, c->stream>>>(geo, lev(0), proj_type, dt, buf(0, hg::kPhi),
                                                              unew, uold, gpi, rhohalf, b0, alt, nc(0));
        launched();
        k_hg_update_pi<<<blocks(nn(0)), kThreads, 0, c->stream>>>(lev(0), proj_type, dt, buf(0, hg::kPhi),
                                                                 pi, nn(0));
        launched();
    }
};

}  // namespace

}  // namespace mac

using namespace mac;

extern "C" {

int mac_hgproject_dense(mac_ctx* c, int proj_type, double dt, int dense_stencil, double rel_eps,
                        double* unew, const double* uold, double* gpi, const double* rhohalf,
                        double* pi, const double* beta0_cart, const double* nodalrhs,
                        mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if (!c || !unew || !gpi || !rhohalf || !pi) return st->status = MAC_ERR_INVALID;
    if (proj_type < hg::kInitial || proj_type > hg::kRegular) return st->status = MAC_ERR_INVALID;
    if (proj_type == hg::kPressureIters && !uold) return st->status = MAC_ERR_INVALID;
    if ((proj_type == hg::kPressureIters || proj_type == hg::kRegular) && !(dt > 0.0))
        return st->status = MAC_ERR_INVALID;
    // the colour-parallel sweeps need even periodic extents (same-colour nodes uncoupled)
    for (int d = 0; d < c->dm; ++d)
        if (c->bc_lo[d] == MAC_BC_PER && (c->n[d] & 1)) return st->status = MAC_ERR_UNSUPPORTED;
    const auto t0 = std::chrono::steady_clock::now();
    begin_call_stats(c, st);
    int rc = hg_ensure(c);
    if (rc) return st->status = rc;
    HgState* H = c->hgs;
    H->geo.dense = dense_stencil ? 1 : 0;
    HgExec ex{c, H, (int)H->L.size(), H->geo, !(H->geo.dlo[0] || H->geo.dhi[0] || H->geo.dlo[1] ||
                                                 H->geo.dhi[1] || H->geo.dlo[2] || H->geo.dhi[2])};
    ex.proj_type = proj_type;
    ex.dt = dt;
    ex.unew = unew;
    ex.uold = uold;
    ex.gpi = gpi;
    ex.rhohalf = rhohalf;
    ex.pi = pi;
    ex.b0 = beta0_cart;
    ex.nodalrhs = nodalrhs;
    ex.alt = (proj_type != hg::kInitial && proj_type != hg::kDivuIters && c->o.use_alt_energy_fix) ? 1 : 0;
    // rhohalf and beta0 must be positive and finite
    if (cudaMemsetAsync(H->flag, 0, sizeof(int), c->stream) != cudaSuccess) rc = MAC_ERR_CUDA;
    if (!rc) {
        k_hg_check<<<blocks_for(H->L[0].nc, c->sms), kThreads, 0, c->stream>>>(rhohalf, beta0_cart, H->flag,
                                                                            H->L[0].nc);
        ex.launched();
        if (cudaMemcpyAsync(H->h_flag, H->flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
            cudaStreamSynchronize(c->stream) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "hg density check", __FILE__, __LINE__);
            rc = MAC_ERR_CUDA;
        }
        if (!rc && ex.err) rc = ex.err;
        if (!rc && *H->h_flag) rc = MAC_ERR_BAD_DENSITY;
    }
    hg::SolveStats S{};
    cudaEventRecord(c->ev[0], c->stream);
    if (!rc) {
        rc = hg::project(ex, rel_eps > 0.0 ? rel_eps : 1e-12, c->o.max_vcycles, c->o.nu1, c->o.nu2, &S);
        if (rc == 1) rc = MAC_ERR_NOT_CONVERGED;
        if (rc == -1) rc = MAC_ERR_NONFINITE;
    }
    cudaEventRecord(c->ev[2], c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess && !rc) {
        set_last_cuda_error(cudaGetLastError(), "cudaStreamSynchronize", __FILE__, __LINE__);
        rc = MAC_ERR_CUDA;
    }
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev[0], c->ev[2]) == cudaSuccess) st->solve_ms = ms;
    cudaGetLastError();
    st->vcycles = S.cycles;
    st->nlevels = (int)H->L.size();
    st->fnorm = S.fnorm;
    st->resid0 = S.resid0;
    st->rel_resid = S.rel_resid;
    st->nhist = S.nhist;
    for (int q = 0; q < S.nhist && q < 64; ++q) st->hist[q] = S.hist[q];
    st->status = rc;
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    end_call_stats(c, st);
    report_call(c, "hgproject_dense", st);
    return rc;
}

}  // extern "C"
