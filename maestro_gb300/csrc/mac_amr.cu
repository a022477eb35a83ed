// Multi-level (AMR) MAC projection on the GPU: the composite cell functions of mac_amr.cuh as
// kernels, the executor that runs amr_solve / amr_project on device arrays, and the C ABI
// (mac_ctx_set_amr, mac_macproject_ml_dense).
//
// Level 0 is the context's own one-level geometry; its multigrid (the FP64 V-cycle of
// mac_solver.cu, with the context's coarsening, tail and bottom solve) is the coarse correction
// of the multi-level cycle.  Finer levels are FP64 arrays over the bounding box of their boxes
// grown by one cell (amr::level_box) with a byte mask (kIn: the level's boxes; kCov: under the
// next finer level): one thread per cell or face of that box, masked.  All launches go to the
// context's stream; the host reads one residual norm per multi-level cycle.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "mac_amr.cuh"
#include "mac_internal.cuh"

namespace mac {

using amr::Geo;
using amr::Lev;

namespace {

constexpr int kThreads = 256;
constexpr int kReduceBlocks = 1024;   // per-level partial slots of the valid-cell reductions
constexpr int kMixedInner = 2;        // FP32 multi-level V-cycles per FP64 step (mixed precision)

// ---- kernels (grid-stride over the cells / faces of one level) --------------------------------

#define AMR_LOOP(N) for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < (N); \
                         idx += (long)gridDim.x * blockDim.x)

template <typename T>
__global__ void k_defect(Geo G, amr::LevT<T> L, amr::LevT<T> C, const T* u, const T* cu,
                         const T* f, T* r, long N) {
    AMR_LOOP(N) amr::defect_cell(G, L, C, idx, u, cu, f, r);
}

// One colour of a sweep: one thread per cell of that colour (N = amr::colour_threads).
template <typename T>
__global__ void k_gsrb(Geo G, amr::LevT<T> L, int colour, T* u, const T* f, long N) {
    AMR_LOOP(N) {
        const long c = amr::colour_cell(L, idx, colour);
        if (c >= 0) amr::gsrb_cell(G, L, c, colour, u, f);
    }
}

template <typename T>
__global__ void k_reflux(Geo G, amr::LevT<T> F, amr::LevT<T> C, const T* uf, const T* uc, T* res,
                         long N) {
    AMR_LOOP(N) amr::reflux_cell(G, F, C, idx, uf, uc, res);
}

template <typename T>
__global__ void k_restrict(Geo G, amr::LevT<T> F, amr::LevT<T> C, const T* fine, T* crse, long N) {
    AMR_LOOP(N) amr::restrict_cell(G, F, C, idx, fine, crse);
}

template <typename T>
__global__ void k_prolong(Geo G, amr::LevT<T> F, amr::LevT<T> C, const T* uc, T* uf, long N) {
    AMR_LOOP(N) amr::prolong_cell(G, F, C, idx, uc, uf);
}

template <typename T>
__global__ void k_axpy3(amr::LevT<T> L, T* uu, const T* hold, const T* du, long N) {
    AMR_LOOP(N) if (amr::in_region(L, idx)) uu[idx] += hold[idx] + du[idx];
}

template <typename T>
__global__ void k_add_region(amr::LevT<T> L, T* phi, const T* uu, long N) {
    AMR_LOOP(N) if (amr::in_region(L, idx)) phi[idx] += uu[idx];
}

// Per-block partials over the cells of one level: [0] sum of vol * x, [1] max |x|, [2] NaN
// count, [3] volume.  valid_only: valid cells (kIn without kCov), else every region cell.
template <typename T>
__global__ void k_reduce(amr::LevT<T> L, const T* x, double vol, int valid_only, double* part,
                         long N) {
    // Only the volume-weighted sum is FP64 arithmetic: the NaN test and the maximum of |x| work
    // on the IEEE bits (for non-negative doubles the unsigned order of the bits is the numeric
    // order), the cells are counted as integers and the volume is vol x count, a float's
    // widening takes the integer pipe: GB300's FP64 pipe is the narrow one.
    __shared__ double s_sum[kThreads / 32], s_vol[kThreads / 32];
    __shared__ unsigned long long s_max[kThreads / 32], s_nan[kThreads / 32];
    double sum = 0.0;
    unsigned long long mx = 0, nan = 0, cnt = 0;
    AMR_LOOP(N) {
        const bool take = valid_only ? amr::is_valid(L, idx) : amr::in_region(L, idx);
        if (!take) continue;
        double a;
        if (std::is_same<T, float>::value)
            a = to_double((float)x[idx]);
        else
            a = (double)x[idx];
        const unsigned long long b = (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull;
        if (b > 0x7ff0000000000000ull) {
            ++nan;
            continue;
        }
        sum = fma(vol, a, sum);
        mx = b > mx ? b : mx;
        ++cnt;
    }
    double v = vol * (double)cnt;
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        const unsigned long long m = __shfl_down_sync(0xffffffffu, mx, o);
        mx = m > mx ? m : mx;
        nan += __shfl_down_sync(0xffffffffu, nan, o);
        v += __shfl_down_sync(0xffffffffu, v, o);
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        s_sum[w] = sum;
        s_max[w] = mx;
        s_nan[w] = nan;
        s_vol[w] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < kThreads / 32; ++q) {
            sum += s_sum[q];
            mx = s_max[q] > mx ? s_max[q] : mx;
            nan += s_nan[q];
            v += s_vol[q];
        }
        double* p = part + 4 * blockIdx.x;
        p[0] = sum;
        p[1] = __longlong_as_double((long long)mx);
        p[2] = (double)nan;
        p[3] = v;
    }
}

// out[0] sum, out[1] max, out[2] NaN count, out[3] volume, out[4] mean = sum / volume; one
// block, fixed order (deterministic).
__global__ void k_reduce_finish(const double* part, int nparts, double* out) {
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

// x -= *m on the valid cells (valid_only) or every region cell.
template <typename T>
__global__ void k_sub_scalar(amr::LevT<T> L, T* x, const double* m, int valid_only, long N) {
    const T v = (T)*m;
    AMR_LOOP(N) {
        const bool take = valid_only ? amr::is_valid(L, idx) : amr::in_region(L, idx);
        if (take) x[idx] -= v;
    }
}

__global__ void k_scale_b0(Geo G, Lev L, int d, double* u, const double* b0, const double* b0e,
                           int mult, long N) {
    AMR_LOOP(N) {
        int f[3];
        amr::face_coords(L, d, idx, f);
        const double bb = amr::beta0_of_face(G, d, f, b0, b0e);
        u[idx] = mult ? u[idx] * bb : u[idx] / bb;
    }
}

__global__ void k_edge_restrict(Geo G, Lev F, Lev C, int d, double* uc, const double* uf, long N) {
    AMR_LOOP(N) amr::edge_restrict_face(G, F, C, d, idx, uc, uf);
}

__global__ void k_divergence(Geo G, Lev L, const double* u0, const double* u1, const double* u2,
                             const double* macrhs, double* rh, long N) {
    AMR_LOOP(N) amr::divergence_cell(G, L, idx, u0, u1, u2, macrhs, rh);
}

__global__ void k_coeff(Geo G, Lev L, int d, const double* rho, const double* b0,
                        const double* b0e, int alt, double* beta, long N) {
    AMR_LOOP(N) amr::coeff_face(G, L, d, idx, rho, b0, b0e, alt, beta);
}

__global__ void k_correct(Geo G, Lev L, Lev C, int d, const double* phi, const double* cphi,
                          const double* beta, double* u, long N) {
    AMR_LOOP(N) amr::correct_face(G, L, C, d, idx, phi, cphi, beta, u);
}

// A density that is not positive and finite on a cell the level's faces read (its region and
// one cell around it along each direction) raises flag[0].
__global__ void k_check_rho(Geo G, Lev L, const double* rho, int* flag, long N) {
    AMR_LOOP(N) {
        int c[3];
        amr::cell_coords(L, idx, c);
        bool used = amr::in_region(L, idx);
        for (int d = 0; d < G.dm && !used; ++d)
            for (int s = -1; s <= 1 && !used; s += 2) {
                const int q = amr::wrap(G, L, d, c[d] + s);
                if (q < 0) continue;
                int p[3] = {c[0], c[1], c[2]};
                p[d] = q;
                used = amr::inside(L, p) && amr::in_region(L, amr::cix(L, p[0], p[1], p[2]));
            }
        if (!used) continue;
        const double v = rho[idx];
        if (!(v > 0.0) || !(v < INFINITY)) atomicExch(flag, 1);
    }
}

// The caller's whole-level-domain arrays <-> the level's box arrays (back: the level's own faces
// and region cells only).
__global__ void k_full_to_box_faces(Lev L, int d, const double* full, double* box, long N) {
    AMR_LOOP(N) box[idx] = full[amr::full_face(L, d, idx)];
}
__global__ void k_full_to_box_cells(Lev L, const double* full, double* box, long N) {
    AMR_LOOP(N) box[idx] = full[amr::full_cell(L, idx)];
}
__global__ void k_box_to_full_faces(Geo G, Lev L, int d, const double* box, double* full, long N) {
    AMR_LOOP(N) {
        int f[3];
        amr::face_coords(L, d, idx, f);
        if (amr::face_in_level(G, L, d, f)) full[amr::full_face(L, d, idx)] = box[idx];
    }
}
__global__ void k_box_to_full_cells(Lev L, const double* box, double* full, long N) {
    AMR_LOOP(N) if (amr::in_region(L, idx)) full[amr::full_cell(L, idx)] = box[idx];
}

__global__ void k_sync_periodic_faces(Geo G, Lev L, int d, double* u, long N) {
    AMR_LOOP(N) amr::sync_periodic_face(G, L, d, idx, u);
}

__global__ void k_to_single(const double* x, float* y, long N) {
    AMR_LOOP(N) amr::to_single_cell(idx, x, y);
}
__global__ void k_accumulate(Lev L, double* phi, const float* e, long N) {
    AMR_LOOP(N) amr::accumulate_cell(L, idx, phi, e);
}

// Caller fabs of one level <-> the level array; blockIdx.y is the fab.
__global__ void k_fabs_gather(Geo G, Lev L, int dir, const amr::FabDesc* T, int with_ghosts,
                              double* level) {
    const amr::FabDesc B = T[blockIdx.y];
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < B.count;
         e += (long)gridDim.x * blockDim.x)
        amr::fab_gather_elem(G, L, dir, B, e, with_ghosts, level);
}

__global__ void k_fabs_scatter(Geo G, Lev L, int dir, const amr::FabDesc* T, const double* level) {
    const amr::FabDesc B = T[blockIdx.y];
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < B.count;
         e += (long)gridDim.x * blockDim.x)
        amr::fab_scatter_elem(G, L, dir, B, e, level);
}

// create_umac_grown: the ghost faces of fine level F's face fabs from F and the next coarser C.
__global__ void k_fabs_grow(Geo G, Lev F, Lev C, int dir, const amr::FabDesc* T, const double* uf,
                            const double* uc) {
    const amr::FabDesc B = T[blockIdx.y];
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < B.count;
         e += (long)gridDim.x * blockDim.x)
        amr::fab_grow_elem(G, F, C, dir, B, e, uf, uc);
}

inline int blocks_for(long n, int sms) {
    const long b = (n + kThreads - 1) / kThreads;
    const long cap = (long)std::max(1, sms) * 16;
    return (int)std::max(1L, std::min(b, cap));
}

}  // namespace

// ---- per-context multi-level state ---------------------------------------------------------------

struct AmrState {
    int nlev = 0;
    Geo geo{};
    // kernel-class timing (mac_opts.timing): CUDA events around the finest level's sweeps, read
    // after the call
    struct Span {
        int cls, launches;
        cudaEvent_t a, b;
    };
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<Span> spans;
    std::vector<std::vector<int>> boxes;   // per level: lo[3], hi[3] per box (level indices)
    struct LevelStore {
        Lev lev{};
        unsigned char* mask = nullptr;
        double* beta[3] = {nullptr, nullptr, nullptr};
        double* buf[amr::kNumBufs] = {};
        // FP32 copy of the level (mixed precision; allocated on first use)
        amr::LevT<float> lev32{};
        float* beta32[3] = {nullptr, nullptr, nullptr};
        float* buf32[amr::kNumBufs] = {};
        double* phi_user = nullptr;   // the caller's phi of this call (aliases buf kPhi)
        long ncell = 0;
    };
    std::vector<LevelStore> L;
    // per-box (fab) calls: level arrays of the inputs, fab tables, host-pointer staging
    struct FabArrays {
        double* u[3] = {nullptr, nullptr, nullptr};
        double* phi = nullptr;
        double* rho = nullptr;
        double* rhs = nullptr;
        double* b0 = nullptr;
        double* b0e = nullptr;
    };
    std::vector<FabArrays> F;
    amr::FabDesc* h_tab = nullptr;   // pinned
    amr::FabDesc* d_tab = nullptr;
    size_t tab_cap = 0;
    double* staging = nullptr;
    size_t staging_cap = 0;
    double* part = nullptr;     // reduction partials: kReduceBlocks * 4 per level
    double* out = nullptr;      // reduction result (5 doubles) + 8 scratch
    double* h_out = nullptr;    // pinned mirror
    int* flag = nullptr;        // device flag (bad density)
    int* h_flag = nullptr;
    std::vector<void*> allocs;
    size_t bytes = 0;
};

void amr_release(mac_ctx* c) {
    AmrState* A = c->amr;
    if (!A) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (void* p : A->allocs) cudaFree(p);
    if (A->staging) cudaFree(A->staging);
    if (A->h_tab) cudaFreeHost(A->h_tab);
    if (A->h_out) cudaFreeHost(A->h_out);
    if (A->h_flag) cudaFreeHost(A->h_flag);
    for (cudaEvent_t e : A->ev_pool) cudaEventDestroy(e);
    delete A;
    c->amr = nullptr;
}

namespace {

template <typename T>
int amr_alloc(AmrState* A, T** p, size_t n) {
    void* q = nullptr;
    const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    if (cudaMalloc(&q, bytes) != cudaSuccess) {
        cudaGetLastError();
        return MAC_ERR_ALLOC;
    }
    A->allocs.push_back(q);
    A->bytes += bytes;
    *p = static_cast<T*>(q);
    return MAC_OK;
}

// Host-side layout check, level boxes and masks (alignment to the ratio 2, boxes inside the level
// domain, proper nesting with one coarse cell of buffer, diagonals included).  Each level's
// arrays cover the bounding box of its boxes grown by one cell (amr::level_box); level 0 the
// domain.
int build_masks(const mac_ctx* c, int nlev, const int* nboxes, const int* box_lo,
                const int* box_hi, std::vector<std::vector<unsigned char>>& masks,
                std::vector<std::vector<int>>& boxes, std::vector<Lev>& geom) {
    const int dm = c->dm;
    masks.assign(nlev, {});
    boxes.assign(nlev, {});
    geom.assign(nlev, Lev{});
    int per[3];
    for (int d = 0; d < 3; ++d) per[d] = d < dm && c->bc_lo[d] == MAC_BC_PER;
    int off = 0;
    for (int l = 0; l < nlev; ++l) {
        Lev& V = geom[l];
        for (int d = 0; d < 3; ++d) {
            V.n[d] = d < dm ? (c->n[d] << l) : 1;
            V.lo[d] = 0;
            V.ext[d] = V.n[d];
        }
        if (l == 0) continue;
        if (nboxes[l] < 1) return MAC_ERR_INVALID;
        int rlo[3] = {1 << 30, 1 << 30, 1 << 30}, rhi[3] = {-1, -1, -1};
        for (int b = 0; b < nboxes[l]; ++b, ++off) {
            int lo[3], hi[3];
            for (int d = 0; d < 3; ++d) {
                lo[d] = box_lo[3 * off + d] - (d < dm ? (c->g.domain_lo[d] << l) : 0);
                hi[d] = box_hi[3 * off + d] - (d < dm ? (c->g.domain_lo[d] << l) : 0);
                if (d >= dm) {
                    if (lo[d] != 0 || hi[d] != 0) return MAC_ERR_INVALID;
                    continue;
                }
                if (lo[d] < 0 || hi[d] >= V.n[d] || hi[d] < lo[d]) return MAC_ERR_INVALID;
                if ((lo[d] & 1) || !(hi[d] & 1)) return MAC_ERR_INVALID;
            }
            for (int d = 0; d < 3; ++d) {
                boxes[l].push_back(lo[d]);
                rlo[d] = std::min(rlo[d], lo[d]);
                rhi[d] = std::max(rhi[d], hi[d]);
            }
            for (int d = 0; d < 3; ++d) boxes[l].push_back(hi[d]);
        }
        amr::level_box(dm, V.n, per, rlo, rhi, V.lo, V.ext);
    }
    for (int l = 0; l < nlev; ++l) {
        const Lev& V = geom[l];
        const long N = amr::ncells(V);
        if (N > (1L << 31)) return MAC_ERR_TOO_LARGE;
        masks[l].assign((size_t)N, l == 0 ? amr::kIn : 0);
        for (size_t q = 0; q + 5 < boxes[l].size(); q += 6)
            for (int k = boxes[l][q + 2]; k <= boxes[l][q + 5]; ++k)
                for (int j = boxes[l][q + 1]; j <= boxes[l][q + 4]; ++j)
                    for (int i = boxes[l][q]; i <= boxes[l][q + 3]; ++i)
                        masks[l][(size_t)amr::cix(V, i, j, k)] = amr::kIn;
    }
    auto wrapq = [&](int l, int d, int q) {
        const int n = geom[l].n[d];
        if (q < 0) return per[d] ? q + n : -1;
        if (q >= n) return per[d] ? q - n : -1;
        return q;
    };
    for (int l = 1; l < nlev; ++l) {
        const Lev& F = geom[l];
        const Lev& K = geom[l - 1];
        for (long idx = 0; idx < amr::ncells(F); ++idx) {
            if (!(masks[l][(size_t)idx] & amr::kIn)) continue;
            int fc[3];
            amr::cell_coords(F, idx, fc);
            const int cc[3] = {dm > 0 ? fc[0] >> 1 : fc[0], dm > 1 ? fc[1] >> 1 : fc[1],
                               dm > 2 ? fc[2] >> 1 : fc[2]};
            if (!amr::inside(K, cc)) return MAC_ERR_INVALID;
            masks[l - 1][(size_t)amr::cix(K, cc[0], cc[1], cc[2])] |= amr::kCov;
            for (int a2 = -(dm > 2); a2 <= (dm > 2); ++a2)
                for (int a1 = -(dm > 1); a1 <= (dm > 1); ++a1)
                    for (int a0 = -1; a0 <= 1; ++a0) {
                        const int q[3] = {wrapq(l - 1, 0, cc[0] + a0), wrapq(l - 1, 1, cc[1] + a1),
                                          wrapq(l - 1, 2, cc[2] + a2)};
                        if (q[0] < 0 || q[1] < 0 || q[2] < 0) continue;
                        if (!amr::inside(K, q) || !(masks[l - 1][(size_t)amr::cix(K, q[0], q[1], q[2])] & amr::kIn))
                            return MAC_ERR_INVALID;
                    }
        }
    }
    return MAC_OK;
}

// The executor of amr_solve / amr_project on the context's stream.
// Level accessors per precision.
template <typename T> struct AmrAccess;
template <> struct AmrAccess<double> {
    static amr::LevT<double> lev(const AmrState::LevelStore& S) { return S.lev; }
    static double*& buf(AmrState::LevelStore& S, int w) { return S.buf[w]; }
};
template <> struct AmrAccess<float> {
    static amr::LevT<float> lev(const AmrState::LevelStore& S) { return S.lev32; }
    static float*& buf(AmrState::LevelStore& S, int w) { return S.buf32[w]; }
};

// The multigrid half of the executor in precision T on the context's stream (FP64; FP32 for the
// inner cycles of the mixed-precision solve, whose level-0 correction is still the FP64
// one-level V-cycle).
template <typename T>
struct GpuMl {
    mac_ctx* c;
    AmrState* A;
    int nlev;
    Geo geo;
    bool singular;
    int err = MAC_OK;

    amr::LevT<T> lev(int l) const { return AmrAccess<T>::lev(A->L[l]); }
    T* buf(int l, int which) const { return AmrAccess<T>::buf(A->L[l], which); }
    long ncell(int l) const { return A->L[l].ncell; }
    int blocks(long n) const { return blocks_for(n, c->sms); }
    void launched() {
        ++c->issued;
        if (!err && cudaPeekAtLastError() != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "amr kernel launch", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
        }
    }
    int error() const { return err; }

    void defect(int l, const T* uu, const T* cu, const T* f, T* r) {
        const amr::LevT<T> C = l ? lev(l - 1) : lev(l);
        k_defect<T><<<blocks(ncell(l)), kThreads, 0, c->stream>>>(geo, lev(l), C, uu, cu, f, r, ncell(l));
        launched();
    }
    cudaEvent_t next_event() {
        if (A->ev_used < A->ev_pool.size()) return A->ev_pool[A->ev_used++];
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "cudaEventCreate", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
            return nullptr;
        }
        A->ev_pool.push_back(e);
        ++A->ev_used;
        return e;
    }
    void gsrb(int l, T* uu, const T* f, int nu) {
        // timing: the finest level's sweeps (one span per call)
        const bool tm = c->o.timing && l == nlev - 1 && !err;
        const long long before = c->issued;
        cudaEvent_t ta = tm ? next_event() : nullptr;
        if (ta) cudaEventRecord(ta, c->stream);
        gsrb_launch(l, uu, f, nu);
        if (ta) {
            cudaEvent_t tb = next_event();
            if (tb) {
                cudaEventRecord(tb, c->stream);
                A->spans.push_back(AmrState::Span{MAC_KT_SMOOTH, (int)(c->issued - before), ta, tb});
            }
        }
    }
    void gsrb_launch(int l, T* uu, const T* f, int nu) {
        for (int s = 0; s < nu; ++s)
            for (int colour = 0; colour < 2; ++colour) {
                const long nt = amr::colour_threads(lev(l));
                k_gsrb<T><<<blocks(nt), kThreads, 0, c->stream>>>(geo, lev(l), colour, uu, f, nt);
                launched();
            }
    }
    void reflux(int l, const T* uf, const T* uc, T* res) {
        k_reflux<T><<<blocks(ncell(l - 1)), kThreads, 0, c->stream>>>(geo, lev(l), lev(l - 1), uf, uc, res, ncell(l - 1));
        launched();
    }
    void restrict_cov(int l, const T* fine, T* crse) {
        k_restrict<T><<<blocks(ncell(l - 1)), kThreads, 0, c->stream>>>(geo, lev(l), lev(l - 1), fine, crse, ncell(l - 1));
        launched();
    }
    void prolong(int l, const T* uc, T* uf) {
        k_prolong<T><<<blocks(ncell(l)), kThreads, 0, c->stream>>>(geo, lev(l), lev(l - 1), uc, uf, ncell(l));
        launched();
    }
    void axpy3(int l, T* uu, const T* hold, const T* du) {
        k_axpy3<T><<<blocks(ncell(l)), kThreads, 0, c->stream>>>(lev(l), uu, hold, du, ncell(l));
        launched();
    }
    void add_region(int l, T* phi, const T* uu) {
        k_add_region<T><<<blocks(ncell(l)), kThreads, 0, c->stream>>>(lev(l), phi, uu, ncell(l));
        launched();
    }
    void zero(int l, T* x) {
        if (!err && cudaMemsetAsync(x, 0, sizeof(T) * ncell(l), c->stream) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "cudaMemsetAsync", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
        }
    }
    void copy(int l, T* dst, const T* src) {
        if (!err && cudaMemcpyAsync(dst, src, sizeof(T) * ncell(l), cudaMemcpyDeviceToDevice,
                                    c->stream) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "cudaMemcpyAsync", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
        }
    }
    void swap_bufs(int l, int a, int b) { std::swap(AmrAccess<T>::buf(A->L[l], a), AmrAccess<T>::buf(A->L[l], b)); }

    // Partials of x over the valid cells (valid_only) or the region cells of level l, appended at
    // slot *nparts of A->part.
    template <typename U>
    void reduce_level(int l, const U* x, int valid_only, int* nparts) {
        const amr::LevT<U> L = AmrAccess<U>::lev(A->L[l]);
        const double vol = L.h[0] * (geo.dm > 1 ? L.h[1] : 1.0) * (geo.dm > 2 ? L.h[2] : 1.0);
        const int nb = std::min(kReduceBlocks, blocks(ncell(l)));
        k_reduce<U><<<nb, kThreads, 0, c->stream>>>(L, x, vol, valid_only, A->part + 4 * *nparts, ncell(l));
        launched();
        *nparts += nb;
    }
    void finish_reduce(int nparts) {
        k_reduce_finish<<<1, kThreads, 0, c->stream>>>(A->part, nparts, A->out);
        launched();
    }
    // Reduce buf(which) over the valid cells of every level into A->out on the device.
    void reduce(int which) {
        int nparts = 0;
        for (int l = 0; l < nlev; ++l) reduce_level<T>(l, buf(l, which), 1, &nparts);
        finish_reduce(nparts);
    }
    bool fetch() {
        if (err) return false;
        if (cudaMemcpyAsync(A->h_out, A->out, 5 * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream) != cudaSuccess ||
            cudaStreamSynchronize(c->stream) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "amr reduction", __FILE__, __LINE__);
            err = MAC_ERR_CUDA;
            return false;
        }
        return true;
    }
    double valid_max(int which) {
        reduce(which);
        if (!fetch()) return NAN;
        return A->h_out[2] > 0.0 ? NAN : A->h_out[1];
    }
    double valid_mean(int which) {
        reduce(which);
        if (!fetch()) return NAN;
        return A->h_out[4];
    }
    void sub_valid(int which, double m) {
        // the mean is still in A->out[4] from valid_mean (same stream, nothing in between)
        (void)m;
        for (int l = 0; l < nlev; ++l) {
            k_sub_scalar<T><<<blocks(ncell(l)), kThreads, 0, c->stream>>>(lev(l), buf(l, which), A->out + 4, 1, ncell(l));
            launched();
        }
    }

    // One FP64 V-cycle of the level-0 multigrid on rhs from a zero guess into e (natural layout);
    // for a singular problem the mean of the right-hand side is removed first and the mean of
    // the correction after (the constant is in the null space of the composite operator).
    int level0_fp64(const double* rhs, double* e) {
        if (err) return err;
        Level& F = c->lev[0];
        double* r0 = A->L[0].buf[amr::kTmp];
        const amr::LevT<double> L0 = A->L[0].lev;
        if (cudaMemcpyAsync(r0, rhs, sizeof(double) * ncell(0), cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
            err = MAC_ERR_CUDA;
        if (!err && singular) {
            int np = 0;
            reduce_level<double>(0, r0, 0, &np);
            finish_reduce(np);
            k_sub_scalar<double><<<blocks(ncell(0)), kThreads, 0, c->stream>>>(L0, r0, A->out + 4, 0, ncell(0));
            launched();
        }
        int rc = err ? err : natural_to_level0(c, r0, F.a64.f);
        if (!rc && cudaMemsetAsync(F.a64.phi, 0, sizeof(double) * (size_t)F.d.ncell, c->stream) != cudaSuccess)
            rc = MAC_ERR_CUDA;
        if (!rc) rc = level0_fp64_vcycle(c);
        if (!rc) rc = level0_to_natural(c, F.a64.phi, e);
        if (!rc && singular) {
            int np = 0;
            reduce_level<double>(0, e, 0, &np);
            finish_reduce(np);
            k_sub_scalar<double><<<blocks(ncell(0)), kThreads, 0, c->stream>>>(L0, e, A->out + 4, 0, ncell(0));
            launched();
        }
        if (rc && !err) err = rc;
        return err;
    }
    // One FP32 V-cycle of the level-0 multigrid (the one-level solver's mixed-precision inner
    // cycle: over-relaxed half-sweeps, its V-cycle shape and exact bottom) on rhs from a zero
    // guess into e, natural layout; the means as in level0_fp64.
    int level0_fp32(const float* rhs, float* e) {
        if (err) return err;
        Level& F = c->lev[0];
        float* r0 = A->L[0].buf32[amr::kTmp];
        const amr::LevT<float> L0 = A->L[0].lev32;
        if (cudaMemcpyAsync(r0, rhs, sizeof(float) * ncell(0), cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
            err = MAC_ERR_CUDA;
        if (!err && singular) {
            int np = 0;
            reduce_level<float>(0, r0, 0, &np);
            finish_reduce(np);
            k_sub_scalar<float><<<blocks(ncell(0)), kThreads, 0, c->stream>>>(L0, r0, A->out + 4, 0, ncell(0));
            launched();
        }
        int rc = err ? err : natural_to_level0(c, r0, F.a32.f);
        if (!rc && cudaMemsetAsync(F.a32.phi, 0, sizeof(float) * (size_t)F.d.ncell, c->stream) != cudaSuccess)
            rc = MAC_ERR_CUDA;
        if (!rc) rc = level0_fp32_vcycle(c);
        if (!rc) rc = level0_to_natural(c, F.a32.phi, e);
        if (!rc && singular) {
            int np = 0;
            reduce_level<float>(0, e, 0, &np);
            finish_reduce(np);
            k_sub_scalar<float><<<blocks(ncell(0)), kThreads, 0, c->stream>>>(L0, e, A->out + 4, 0, ncell(0));
            launched();
        }
        if (rc && !err) err = rc;
        return err;
    }
    int level0_correction(const T* rhs, T* e) {
        if constexpr (std::is_same<T, double>::value) {
            return level0_fp64(rhs, e);
        } else {
            return level0_fp32(rhs, e);
        }
    }
};

// The FP64 executor: the multigrid, the projection steps, and the hand-over to the FP32 cycles.
struct GpuExec : GpuMl<double> {
    // this call's inputs (device pointers, level-domain arrays)
    double* const* u = nullptr;            // [3 l + d]
    const double* const* rho = nullptr;
    const double* const* macrhs = nullptr;
    const double* const* b0 = nullptr;
    const double* const* b0e = nullptr;
    int alt = 0;

    int prepare_level0() {
        if (err) return err;
        int rc = set_call_state(c, false);
        if (!rc) rc = set_otf_mode(c, false);
        if (!rc) rc = setup_fine_from_faces(c, A->L[0].beta[0], A->L[0].beta[1],
                                            geo.dm == 3 ? A->L[0].beta[2] : nullptr, nullptr);
        // mixed precision: the FP32 level-0 operator of the inner cycles' coarse correction
        if (!rc && c->o.precision == MAC_PREC_MIXED) rc = setup_fp32_copies(c);
        if (!rc) rc = setup_coarse_levels(c);
        singular = c->singular;
        return rc;
    }
    void faces_to_single() {
        for (int l = 0; l < nlev; ++l)
            for (int d = 0; d < geo.dm; ++d) {
                const long nf = amr::nfaces(lev(l), d);
                k_to_single<<<blocks(nf), kThreads, 0, c->stream>>>(A->L[l].beta[d], A->L[l].beta32[d], nf);
                launched();
            }
    }
    void to_single(int l, const double* x, float* y) {
        k_to_single<<<blocks(ncell(l)), kThreads, 0, c->stream>>>(x, y, ncell(l));
        launched();
    }
    void accumulate(int l, double* phi, const float* e) {
        k_accumulate<<<blocks(ncell(l)), kThreads, 0, c->stream>>>(lev(l), phi, e, ncell(l));
        launched();
    }

    // ---- projection steps ----
    void scale_b0(int l, bool mult) {
        if (!b0) return;
        for (int d = 0; d < geo.dm; ++d) {
            const long nf = amr::nfaces(lev(l), d);
            k_scale_b0<<<blocks(nf), kThreads, 0, c->stream>>>(geo, lev(l), d, u[3 * l + d], b0[l], b0e[l], mult ? 1 : 0, nf);
            launched();
        }
    }
    void edge_restrict(int l) {
        for (int d = 0; d < geo.dm; ++d) {
            const long nf = amr::nfaces(lev(l - 1), d);
            k_edge_restrict<<<blocks(nf), kThreads, 0, c->stream>>>(geo, lev(l), lev(l - 1), d, u[3 * (l - 1) + d], u[3 * l + d], nf);
            launched();
        }
    }
    void divergence(int l) {
        k_divergence<<<blocks(ncell(l)), kThreads, 0, c->stream>>>(
            geo, lev(l), u[3 * l], u[3 * l + 1], geo.dm == 3 ? u[3 * l + 2] : nullptr,
            macrhs ? macrhs[l] : nullptr, buf(l, amr::kRh), ncell(l));
        launched();
    }
    void coeffs(int l) {
        for (int d = 0; d < geo.dm; ++d) {
            const long nf = amr::nfaces(lev(l), d);
            k_coeff<<<blocks(nf), kThreads, 0, c->stream>>>(geo, lev(l), d, rho[l], b0 ? b0[l] : nullptr,
                                                            b0 ? b0e[l] : nullptr, alt, A->L[l].beta[d], nf);
            launched();
        }
    }
    void correct(int l) {
        const Lev C = l ? lev(l - 1) : lev(l);
        const double* cphi = l ? buf(l - 1, amr::kPhi) : nullptr;
        for (int d = 0; d < geo.dm; ++d) {
            const long nf = amr::nfaces(lev(l), d);
            k_correct<<<blocks(nf), kThreads, 0, c->stream>>>(geo, lev(l), C, d, buf(l, amr::kPhi), cphi,
                                                              A->L[l].beta[d], u[3 * l + d], nf);
            launched();
        }
    }
};

}  // namespace

int amr_configure(mac_ctx* c, int nlev, const int* nboxes, const int* box_lo, const int* box_hi) {
    if (nlev < 2 || nlev > amr::kMaxLevels || !nboxes || !box_lo || !box_hi) return MAC_ERR_INVALID;
    std::vector<std::vector<unsigned char>> masks;
    std::vector<std::vector<int>> boxes;
    std::vector<Lev> geom;
    int rc = build_masks(c, nlev, nboxes, box_lo, box_hi, masks, boxes, geom);
    if (rc) return rc;
    amr_release(c);
    AmrState* A = new AmrState();
    c->amr = A;
    A->nlev = nlev;
    A->boxes = boxes;
    Geo& G = A->geo;
    G.dm = c->dm;
    G.va = c->dm - 1;
    for (int d = 0; d < 3; ++d) {
        G.per[d] = c->bc_lo[d] == MAC_BC_PER;
        G.dlo[d] = c->bc_lo[d] == MAC_BC_DIR;
        G.dhi[d] = c->bc_hi[d] == MAC_BC_DIR;
    }
    A->L.assign(nlev, AmrState::LevelStore());
    for (int l = 0; l < nlev && !rc; ++l) {
        AmrState::LevelStore& S = A->L[l];
        for (int d = 0; d < 3; ++d) {
            S.lev.n[d] = geom[l].n[d];
            S.lev.lo[d] = geom[l].lo[d];
            S.lev.ext[d] = geom[l].ext[d];
            amr::set_spacing(S.lev, d, d < c->dm ? c->dx[d] / (double)(1 << l) : c->dx[d]);
        }
        const long N = amr::ncells(S.lev);
        S.ncell = N;
        rc = amr_alloc(A, &S.mask, (size_t)N);
        for (int d = 0; d < c->dm && !rc; ++d) rc = amr_alloc(A, &S.beta[d], (size_t)amr::nfaces(S.lev, d));
        for (int b = 0; b < amr::kNumBufs && !rc; ++b) rc = amr_alloc(A, &S.buf[b], (size_t)N);
        if (rc) break;
        if (cudaMemcpy(S.mask, masks[l].data(), (size_t)N, cudaMemcpyHostToDevice) != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "cudaMemcpy(mask)", __FILE__, __LINE__);
            rc = MAC_ERR_CUDA;
            break;
        }
        S.lev.mask = S.mask;
        for (int d = 0; d < 3; ++d) S.lev.b[d] = S.beta[d];
    }
    if (!rc) rc = amr_alloc(A, &A->part, (size_t)4 * kReduceBlocks * nlev);
    if (!rc) rc = amr_alloc(A, &A->out, 16);
    if (!rc) rc = amr_alloc(A, &A->flag, 1);
    if (!rc && (cudaMallocHost((void**)&A->h_out, 16 * sizeof(double)) != cudaSuccess ||
                cudaMallocHost((void**)&A->h_flag, sizeof(int)) != cudaSuccess)) {
        cudaGetLastError();
        rc = MAC_ERR_ALLOC;
    }
    if (rc) amr_release(c);
    return rc;
}

// FP32 copies of the levels for the mixed-precision solve (allocated on first use).
int amr_ensure_single(mac_ctx* c) {
    AmrState* A = c->amr;
    if (A->L[0].buf32[0]) return MAC_OK;
    for (AmrState::LevelStore& S : A->L) {
        int rc = MAC_OK;
        for (int d = 0; d < c->dm && !rc; ++d) rc = amr_alloc(A, &S.beta32[d], (size_t)amr::nfaces(S.lev, d));
        for (int b = 0; b < amr::kNumBufs && !rc; ++b) rc = amr_alloc(A, &S.buf32[b], (size_t)S.ncell);
        if (rc) return rc;
        for (int d = 0; d < 3; ++d) {
            S.lev32.n[d] = S.lev.n[d];
            S.lev32.lo[d] = S.lev.lo[d];
            S.lev32.ext[d] = S.lev.ext[d];
            amr::set_spacing(S.lev32, d, S.lev.h[d]);
            S.lev32.b[d] = S.beta32[d];
        }
        S.lev32.mask = S.lev.mask;
    }
    return MAC_OK;
}

// The multi-level projection on level arrays already on the device (the caller's, or gathered
// from fabs); fills the solve fields of *st and returns the status code.
int ml_core(mac_ctx* c, double* const* umac, double* const* phi, const double* const* rho,
            const double* const* macrhs, const double* const* beta0,
            const double* const* beta0_edge, mac_stats* st) {
    AmrState* A = c->amr;
    const int nl = A->nlev;
    GpuExec ex;
    ex.c = c;
    ex.A = A;
    ex.nlev = nl;
    ex.geo = A->geo;
    ex.singular = c->geom_singular;
    ex.u = umac;
    ex.rho = rho;
    ex.macrhs = macrhs;
    ex.b0 = beta0;
    ex.b0e = beta0_edge;
    ex.alt = c->o.use_alt_energy_fix;
    // phi of this call stands in for the solution buffers
    double* saved_phi[amr::kMaxLevels];
    for (int l = 0; l < nl; ++l) {
        saved_phi[l] = A->L[l].buf[amr::kPhi];
        A->L[l].buf[amr::kPhi] = phi[l];
    }
    int rc = MAC_OK;
    // densities a level's faces read must be positive and finite
    if (cudaMemsetAsync(A->flag, 0, sizeof(int), c->stream) != cudaSuccess) rc = MAC_ERR_CUDA;
    for (int l = 0; l < nl && !rc; ++l) {
        k_check_rho<<<blocks_for(A->L[l].ncell, c->sms), kThreads, 0, c->stream>>>(
            A->geo, A->L[l].lev, rho[l], A->flag, A->L[l].ncell);
        ex.launched();
    }
    if (!rc && (cudaMemcpyAsync(A->h_flag, A->flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                cudaStreamSynchronize(c->stream) != cudaSuccess)) {
        set_last_cuda_error(cudaGetLastError(), "density check", __FILE__, __LINE__);
        rc = MAC_ERR_CUDA;
    }
    if (!rc && ex.err) rc = ex.err;
    if (!rc && *A->h_flag) rc = MAC_ERR_BAD_DENSITY;
    // MAESTRO's tolerance for nlevs levels: min(eps_mac * 10^(nlevs-1), eps_mac_max)
    // (Source/macproject.f90:217), with the context's rel_eps as eps_mac
    double rel = c->o.rel_eps;
    if (rel < 1e-8) rel = std::min(rel * std::pow(10.0, nl - 1), 1e-8);
    amr::SolveStats S{};
    A->spans.clear();
    A->ev_used = 0;
    cudaEventRecord(c->ev[0], c->stream);
    if (!rc) {
        if (c->o.precision == MAC_PREC_MIXED) {
            // FP32 multi-level cycles (kMixedInner per FP64 step) under FP64 refinement
            rc = amr_ensure_single(c);
            GpuMl<float> ex32;
            ex32.c = c;
            ex32.A = A;
            ex32.nlev = nl;
            ex32.geo = A->geo;
            ex32.singular = c->geom_singular;
            if (!rc)
                rc = amr::amr_project(ex, rel, c->o.abs_eps, c->o.max_vcycles, c->o.nu1, c->o.nu2,
                                      &S, &ex32, kMixedInner);
        } else {
            rc = amr::amr_project(ex, rel, c->o.abs_eps, c->o.max_vcycles, c->o.nu1, c->o.nu2, &S);
        }
        if (rc == 1) rc = MAC_ERR_NOT_CONVERGED;
        if (rc == -1 && S.status == -1) rc = MAC_ERR_NONFINITE;
        if (rc == MAC_OK && std::isnan(S.rel_resid)) rc = MAC_ERR_NONFINITE;
    }
    cudaEventRecord(c->ev[2], c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess && !rc) {
        set_last_cuda_error(cudaGetLastError(), "cudaStreamSynchronize", __FILE__, __LINE__);
        rc = MAC_ERR_CUDA;
    }
    for (int l = 0; l < nl; ++l) A->L[l].buf[amr::kPhi] = saved_phi[l];
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev[0], c->ev[2]) == cudaSuccess) st->solve_ms = ms;
    for (const AmrState::Span& sp : A->spans) {   // timing: the finest level's sweeps
        float t = 0.f;
        if (cudaEventElapsedTime(&t, sp.a, sp.b) != cudaSuccess) continue;
        c->ktime_ms[sp.cls] += t;
        c->ktime_launches[sp.cls] += sp.launches;
    }
    A->spans.clear();
    A->ev_used = 0;
    cudaGetLastError();
    st->vcycles = S.cycles;
    st->fnorm = S.fnorm;
    st->resid0 = S.resid0;
    st->rel_resid = S.rel_resid;
    st->nhist = S.nhist;
    for (int q = 0; q < S.nhist && q < 64; ++q) st->hist[q] = S.hist[q];
    return rc;
}


namespace {

int fab_boxes(const mac_ctx* c, int l) {
    return l == 0 ? c->g.nboxes : (int)(c->amr->boxes[l].size() / 6);
}

// Descriptor of box b of level l as a fab with ng ghosts (dir: face direction, -1 cells).
amr::FabDesc fab_desc(const mac_ctx* c, int l, int b, int dir, int ng) {
    amr::FabDesc D{};
    long cnt = 1;
    for (int d = 0; d < 3; ++d) {
        if (d >= c->dm) {
            D.lo[d] = D.hi[d] = 0;
            D.ext[d] = 1;
            continue;
        }
        if (l == 0) {
            D.lo[d] = c->box_lo[3 * b + d] - c->g.domain_lo[d];
            D.hi[d] = c->box_hi[3 * b + d] - c->g.domain_lo[d];
        } else {
            D.lo[d] = c->amr->boxes[l][6 * b + d];
            D.hi[d] = c->amr->boxes[l][6 * b + 3 + d];
        }
        D.ext[d] = D.hi[d] - D.lo[d] + 1 + (dir == d ? 1 : 0) + 2 * ng;
        cnt *= D.ext[d];
    }
    D.ng = ng;
    D.count = cnt;
    return D;
}

template <typename T>
int grow_device(T** p, size_t* cap, size_t need) {
    if (need <= *cap) return MAC_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    if (cudaMalloc((void**)p, need * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return MAC_ERR_ALLOC;
    }
    *cap = need;
    return MAC_OK;
}

int ensure_fab_arrays(mac_ctx* c, bool rhs, bool b0) {
    AmrState* A = c->amr;
    if (A->F.size() != (size_t)A->nlev) A->F.assign(A->nlev, AmrState::FabArrays());
    for (int l = 0; l < A->nlev; ++l) {
        AmrState::FabArrays& F = A->F[l];
        const Lev& L = A->L[l].lev;
        const long N = A->L[l].ncell;
        int rc = MAC_OK;
        for (int d = 0; d < c->dm && !rc; ++d)
            if (!F.u[d]) rc = amr_alloc(A, &F.u[d], (size_t)amr::nfaces(L, d));
        if (!rc && !F.phi) rc = amr_alloc(A, &F.phi, (size_t)N);
        if (!rc && !F.rho) rc = amr_alloc(A, &F.rho, (size_t)N);
        if (!rc && rhs && !F.rhs) rc = amr_alloc(A, &F.rhs, (size_t)N);
        const int nr = L.n[c->dm - 1];
        if (!rc && b0 && !F.b0) rc = amr_alloc(A, &F.b0, (size_t)nr);
        if (!rc && b0 && !F.b0e) rc = amr_alloc(A, &F.b0e, (size_t)nr + 1);
        if (rc) return rc;
    }
    return MAC_OK;
}

}  // namespace

// Per-box entry: gather the caller's fabs into the level arrays, project, scatter back.
int ml_fabs(mac_ctx* c, int ptr_kind, double* const* umac, int ng_u, double* const* phi,
            int ng_phi, const double* const* rho, int ng_rho, int rho_comp,
            const double* const* macrhs, int ng_rhs, const double* beta0,
            const double* beta0_edge, mac_stats* st) {
    AmrState* A = c->amr;
    const int nl = A->nlev;
    const int dm = c->dm;
    const bool host = ptr_kind == MAC_PTR_HOST;
    int rc = ensure_fab_arrays(c, macrhs != nullptr, beta0 != nullptr);
    if (rc) return rc;
    // tables and staging
    size_t ntab = 0, nstage = 0;
    for (int l = 0; l < nl; ++l) {
        const int nb = fab_boxes(c, l);
        ntab += (size_t)nb * (dm + 3);
        for (int b = 0; b < nb; ++b) {
            for (int d = 0; d < dm; ++d) nstage += (size_t)fab_desc(c, l, b, d, ng_u).count;
            nstage += (size_t)fab_desc(c, l, b, -1, ng_phi).count;
            nstage += (size_t)fab_desc(c, l, b, -1, ng_rho).count;
            if (macrhs) nstage += (size_t)fab_desc(c, l, b, -1, ng_rhs).count;
        }
    }
    if (ntab > A->tab_cap) {
        MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
        if (A->h_tab) cudaFreeHost(A->h_tab);
        if (A->d_tab) cudaFree(A->d_tab);
        A->h_tab = nullptr;
        A->d_tab = nullptr;
        A->tab_cap = 0;
        if (cudaMallocHost((void**)&A->h_tab, ntab * sizeof(amr::FabDesc)) != cudaSuccess ||
            cudaMalloc((void**)&A->d_tab, ntab * sizeof(amr::FabDesc)) != cudaSuccess) {
            cudaGetLastError();
            return MAC_ERR_ALLOC;
        }
        A->tab_cap = ntab;
    }
    if (host) {
        MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
        rc = grow_device(&A->staging, &A->staging_cap, nstage);
        if (rc) return rc;
    }
    size_t tcur = 0, scur = 0;
    std::vector<size_t> tab_u(nl * 3), tab_phi(nl);
    // one array of one level: descriptors, host copies, table upload, gather kernel
    auto gather = [&](int l, int dir, int ng, const double* const* ptrs, long comp_stride_comp,
                      int with_ghosts, double* level, size_t* tab_at) -> int {
        const int nb = fab_boxes(c, l);
        amr::FabDesc* H = A->h_tab + tcur;
        long maxc = 1;
        for (int b = 0; b < nb; ++b) {
            amr::FabDesc D = fab_desc(c, l, b, dir, ng);
            const double* src = ptrs[b] + D.count * comp_stride_comp;
            if (host) {
                double* region = A->staging + scur;
                scur += (size_t)D.count;
                MAC_CUDA_TRY(cudaMemcpyAsync(region, src, (size_t)D.count * sizeof(double),
                                             cudaMemcpyHostToDevice, c->stream));
                D.src = region;
                D.dst = region;
            } else {
                D.src = src;
                D.dst = const_cast<double*>(src);
            }
            H[b] = D;
            maxc = std::max(maxc, D.count);
        }
        MAC_CUDA_TRY(cudaMemcpyAsync(A->d_tab + tcur, H, (size_t)nb * sizeof(amr::FabDesc),
                                     cudaMemcpyHostToDevice, c->stream));
        const dim3 grid((unsigned)std::min<long>((maxc + kThreads - 1) / kThreads, 1024), (unsigned)nb);
        k_fabs_gather<<<grid, kThreads, 0, c->stream>>>(A->geo, A->L[l].lev, dir, A->d_tab + tcur,
                                                       with_ghosts, level);
        MAC_CUDA_TRY(cudaGetLastError());
        ++c->issued;
        if (tab_at) *tab_at = tcur;
        tcur += (size_t)nb;
        return MAC_OK;
    };
    int uoff = 0, boff = 0;
    size_t roff = 0;
    std::vector<double*> up(3 * nl, nullptr), pp(nl), rp(nl), mp(nl), b0p(nl), b0ep(nl);
    for (int l = 0; l < nl && !rc; ++l) {
        const int nb = fab_boxes(c, l);
        AmrState::FabArrays& F = A->F[l];
        for (int d = 0; d < dm && !rc; ++d) {
            rc = gather(l, d, ng_u, umac + uoff + d * nb, 0, 0, F.u[d], &tab_u[3 * l + d]);
            up[3 * l + d] = F.u[d];
        }
        if (!rc) rc = gather(l, -1, ng_phi, phi + boff, 0, 0, F.phi, &tab_phi[l]);
        if (!rc) rc = gather(l, -1, ng_rho, rho + boff, rho_comp, 1, F.rho, nullptr);
        if (!rc && macrhs) rc = gather(l, -1, ng_rhs, macrhs + boff, 0, 0, F.rhs, nullptr);
        pp[l] = F.phi;
        rp[l] = F.rho;
        mp[l] = F.rhs;
        if (!rc && beta0) {
            const size_t nr = (size_t)A->L[l].lev.n[dm - 1];
            if (host) {
                MAC_CUDA_TRY(cudaMemcpyAsync(F.b0, beta0 + roff, nr * sizeof(double),
                                             cudaMemcpyHostToDevice, c->stream));
                MAC_CUDA_TRY(cudaMemcpyAsync(F.b0e, beta0_edge + roff + l, (nr + 1) * sizeof(double),
                                             cudaMemcpyHostToDevice, c->stream));
                b0p[l] = F.b0;
                b0ep[l] = F.b0e;
            } else {
                b0p[l] = const_cast<double*>(beta0 + roff);
                b0ep[l] = const_cast<double*>(beta0_edge + roff + l);
            }
            roff += nr;
        }
        uoff += dm * nb;
        boff += nb;
    }
    if (rc) return rc;
    // the periodic image copy of a fine level's domain-face velocities (only one copy is owned)
    for (int l = 1; l < nl; ++l) {
        const Lev& L = A->L[l].lev;
        for (int d = 0; d < dm; ++d) {
            if (!A->geo.per[d] || L.lo[d] != 0 || L.ext[d] != L.n[d]) continue;
            const long nt = A->L[l].ncell / L.ext[d];
            k_sync_periodic_faces<<<blocks_for(nt, c->sms), kThreads, 0, c->stream>>>(A->geo, L, d, A->F[l].u[d], nt);
            MAC_CUDA_TRY(cudaGetLastError());
            ++c->issued;
        }
    }
    const int solve_rc = ml_core(c, up.data(), pp.data(), rp.data(), macrhs ? mp.data() : nullptr,
                                 beta0 ? b0p.data() : nullptr, beta0 ? b0ep.data() : nullptr, st);
    if (solve_rc != MAC_OK && solve_rc != MAC_ERR_NOT_CONVERGED) return solve_rc;
    // scatter umac and phi back (the tables of the gathers carry dst)
    for (int l = 0; l < nl; ++l) {
        const int nb = fab_boxes(c, l);
        long maxu = 1, maxp = 1;
        for (int b = 0; b < nb; ++b) {
            for (int d = 0; d < dm; ++d) maxu = std::max(maxu, A->h_tab[tab_u[3 * l + d] + b].count);
            maxp = std::max(maxp, A->h_tab[tab_phi[l] + b].count);
        }
        for (int d = 0; d < dm; ++d) {
            const dim3 grid((unsigned)std::min<long>((maxu + kThreads - 1) / kThreads, 1024), (unsigned)nb);
            k_fabs_scatter<<<grid, kThreads, 0, c->stream>>>(A->geo, A->L[l].lev, d,
                                                            A->d_tab + tab_u[3 * l + d], A->F[l].u[d]);
            MAC_CUDA_TRY(cudaGetLastError());
            ++c->issued;
            // the fine levels' ghost faces, as create_umac_grown fills them after the projection
            // (Source/macproject.f90:264-272; the coarsest level's ghosts are left alone there)
            if (l >= 1 && ng_u >= 1) {
                k_fabs_grow<<<grid, kThreads, 0, c->stream>>>(A->geo, A->L[l].lev, A->L[l - 1].lev, d,
                                                             A->d_tab + tab_u[3 * l + d], A->F[l].u[d],
                                                             A->F[l - 1].u[d]);
                MAC_CUDA_TRY(cudaGetLastError());
                ++c->issued;
            }
        }
        const dim3 grid((unsigned)std::min<long>((maxp + kThreads - 1) / kThreads, 1024), (unsigned)nb);
        k_fabs_scatter<<<grid, kThreads, 0, c->stream>>>(A->geo, A->L[l].lev, -1,
                                                        A->d_tab + tab_phi[l], A->F[l].phi);
        MAC_CUDA_TRY(cudaGetLastError());
        ++c->issued;
    }
    if (host) {
        uoff = 0;
        boff = 0;
        for (int l = 0; l < nl; ++l) {
            const int nb = fab_boxes(c, l);
            for (int d = 0; d < dm; ++d)
                for (int b = 0; b < nb; ++b) {
                    const amr::FabDesc& D = A->h_tab[tab_u[3 * l + d] + b];
                    MAC_CUDA_TRY(cudaMemcpyAsync(umac[uoff + d * nb + b], D.src,
                                                 (size_t)D.count * sizeof(double),
                                                 cudaMemcpyDeviceToHost, c->stream));
                }
            for (int b = 0; b < nb; ++b) {
                const amr::FabDesc& D = A->h_tab[tab_phi[l] + b];
                MAC_CUDA_TRY(cudaMemcpyAsync(phi[boff + b], D.src, (size_t)D.count * sizeof(double),
                                             cudaMemcpyDeviceToHost, c->stream));
            }
            uoff += dm * nb;
            boff += nb;
        }
    }
    MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return solve_rc;
}


// Whole-level-domain entry: the caller's arrays are copied into the levels' box arrays, projected,
// and the levels' own faces and region cells copied back.
int ml_dense(mac_ctx* c, double* const* umac, double* const* phi, const double* const* rho,
             const double* const* macrhs, const double* const* beta0,
             const double* const* beta0_edge, mac_stats* st) {
    AmrState* A = c->amr;
    const int nl = A->nlev;
    const int dm = c->dm;
    int rc = ensure_fab_arrays(c, macrhs != nullptr, false);
    if (rc) return rc;
    std::vector<double*> up(3 * nl, nullptr), pp(nl), rp(nl), mp(nl, nullptr);
    auto launched = [&]() -> int {
        ++c->issued;
        if (cudaPeekAtLastError() != cudaSuccess) {
            set_last_cuda_error(cudaGetLastError(), "amr copy launch", __FILE__, __LINE__);
            return MAC_ERR_CUDA;
        }
        return MAC_OK;
    };
    for (int l = 0; l < nl && !rc; ++l) {
        AmrState::FabArrays& F = A->F[l];
        const Lev L = A->L[l].lev;
        const long N = A->L[l].ncell;
        for (int d = 0; d < dm && !rc; ++d) {
            const long nf = amr::nfaces(L, d);
            k_full_to_box_faces<<<blocks_for(nf, c->sms), kThreads, 0, c->stream>>>(L, d, umac[3 * l + d], F.u[d], nf);
            rc = launched();
            up[3 * l + d] = F.u[d];
        }
        k_full_to_box_cells<<<blocks_for(N, c->sms), kThreads, 0, c->stream>>>(L, rho[l], F.rho, N);
        if (!rc) rc = launched();
        k_full_to_box_cells<<<blocks_for(N, c->sms), kThreads, 0, c->stream>>>(L, phi[l], F.phi, N);
        if (!rc) rc = launched();
        if (macrhs && macrhs[l]) {
            k_full_to_box_cells<<<blocks_for(N, c->sms), kThreads, 0, c->stream>>>(L, macrhs[l], F.rhs, N);
            if (!rc) rc = launched();
            mp[l] = F.rhs;
        }
        pp[l] = F.phi;
        rp[l] = F.rho;
    }
    if (rc) return rc;
    const int solve_rc = ml_core(c, up.data(), pp.data(), rp.data(), macrhs ? mp.data() : nullptr,
                                 beta0, beta0_edge, st);
    if (solve_rc != MAC_OK && solve_rc != MAC_ERR_NOT_CONVERGED) return solve_rc;
    for (int l = 0; l < nl && !rc; ++l) {
        AmrState::FabArrays& F = A->F[l];
        const Lev L = A->L[l].lev;
        const long N = A->L[l].ncell;
        for (int d = 0; d < dm && !rc; ++d) {
            const long nf = amr::nfaces(L, d);
            k_box_to_full_faces<<<blocks_for(nf, c->sms), kThreads, 0, c->stream>>>(A->geo, L, d, F.u[d], umac[3 * l + d], nf);
            rc = launched();
        }
        k_box_to_full_cells<<<blocks_for(N, c->sms), kThreads, 0, c->stream>>>(L, F.phi, phi[l], N);
        if (!rc) rc = launched();
    }
    if (!rc) MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return rc ? rc : solve_rc;
}
}  // namespace mac

using namespace mac;

extern "C" {

int mac_ctx_set_amr(mac_ctx* c, int nlev, const int* nboxes, const int* box_lo, const int* box_hi) {
    if (!c) return MAC_ERR_INVALID;
    if (nlev == 1) {
        amr_release(c);
        return MAC_OK;
    }
    return amr_configure(c, nlev, nboxes, box_lo, box_hi);
}

int mac_macproject_ml_dense(mac_ctx* c, double* const* umac, double* const* phi,
                            const double* const* rho, const double* const* macrhs,
                            const double* const* beta0, const double* const* beta0_edge,
                            mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if (!c || !c->amr || !umac || !phi || !rho) return st->status = MAC_ERR_INVALID;
    if ((beta0 == nullptr) != (beta0_edge == nullptr)) return st->status = MAC_ERR_INVALID;
    AmrState* A = c->amr;
    const int nl = A->nlev;
    for (int l = 0; l < nl; ++l) {
        if (!phi[l] || !rho[l]) return st->status = MAC_ERR_INVALID;
        for (int d = 0; d < c->dm; ++d)
            if (!umac[3 * l + d]) return st->status = MAC_ERR_INVALID;
        if (beta0 && (!beta0[l] || !beta0_edge[l])) return st->status = MAC_ERR_INVALID;
    }
    const auto t0 = std::chrono::steady_clock::now();
    begin_call_stats(c, st);
    const int rc = ml_dense(c, umac, phi, rho, macrhs, beta0, beta0_edge, st);
    st->status = rc;
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    end_call_stats(c, st);
    report_call(c, "macproject_ml_dense", st);
    return rc;
}


int mac_macproject_ml(mac_ctx* c, int ptr_kind, double* const* umac, int ng_u,
                      double* const* phi, int ng_phi, const double* const* rho, int ng_rho,
                      int rho_ncomp, int rho_comp, const double* const* macrhs, int ng_rhs,
                      const double* beta0, const double* beta0_edge, mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if (!c || !c->amr || !umac || !phi || !rho) return st->status = MAC_ERR_INVALID;
    if (ptr_kind != MAC_PTR_HOST && ptr_kind != MAC_PTR_DEVICE) return st->status = MAC_ERR_INVALID;
    if (ng_u < 0 || ng_phi < 0 || ng_rho < 1 || ng_rhs < 0) return st->status = MAC_ERR_INVALID;
    if (rho_ncomp < 1 || rho_comp < 0 || rho_comp >= rho_ncomp) return st->status = MAC_ERR_INVALID;
    if ((beta0 == nullptr) != (beta0_edge == nullptr)) return st->status = MAC_ERR_INVALID;
    AmrState* A = c->amr;
    int uoff = 0, boff = 0;
    for (int l = 0; l < A->nlev; ++l) {
        const int nb = fab_boxes(c, l);
        for (int b = 0; b < nb; ++b) {
            if (!phi[boff + b] || !rho[boff + b] || (macrhs && !macrhs[boff + b]))
                return st->status = MAC_ERR_INVALID;
            for (int d = 0; d < c->dm; ++d)
                if (!umac[uoff + d * nb + b]) return st->status = MAC_ERR_INVALID;
        }
        uoff += c->dm * nb;
        boff += nb;
    }
    const auto t0 = std::chrono::steady_clock::now();
    begin_call_stats(c, st);
    const int rc = ml_fabs(c, ptr_kind, umac, ng_u, phi, ng_phi, rho, ng_rho, rho_comp, macrhs,
                           ng_rhs, beta0, beta0_edge, st);
    st->status = rc;
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    end_call_stats(c, st);
    report_call(c, "macproject_ml", st);
    return rc;
}

}  // extern "C"
