// Internal declarations of the GB300 MAC-projection library (not part of the C ABI).
//
// Device layout
// -------------
// Every multigrid level except the coarsest stores its cell fields in a "checkerboard-split"
// layout: the cells of colour c = (i+j+k) & 1 of a level with n0 x n1 x n2 cells live in the
// half-array [c*half, (c+1)*half), half = n0*n1*n2/2, at index h + (n0/2)*(j + n1*k) with
// h = i >> 1.  A red/black Gauss-Seidel half-sweep then reads only the other colour's half and
// writes only its own, both fully coalesced, and the two children of a coarse cell along x sit
// at the same h in the two halves.  The coarsest level (bottom solve) uses the natural layout
// i + n0*(j + n1*k).
//
// Face coefficients are stored per cell as the coefficient of its LOW face, pre-divided by h^2
// (beta'_d = beta_d / h_d^2).  The high face of cell i is the low face of cell i+1.  All
// neighbour indices wrap around (periodic arithmetic in every direction); a non-periodic wall
// stores a zero coefficient on the low face of cell 0, which then also serves as the high face
// of cell n-1 through the wrap.  So one branch-free 7-point kernel covers periodic, Neumann and
// Dirichlet boundaries: Dirichlet faces add 2*beta'_wall to the diagonal only (linear ghost
// phi_g = -phi_0), Neumann faces add nothing.
//
// 2-D problems (nx, ny) are stored as 3-D (nx, ny, 1) with zero z coefficients; the vertical
// direction (beta0 index) is then y.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "maestro_mac.h"

namespace mac {

constexpr int kMaxLevels = 32;
constexpr int kBottomMaxCells = 65536;   // single-CTA bottom solver limit

#define MAC_CUDA_TRY(expr)                                   \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) {                             \
            mac::set_last_cuda_error(_e, #expr, __FILE__, __LINE__); \
            return MAC_ERR_CUDA;                             \
        }                                                    \
    } while (0)

void set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line);

// Dimensions of a level as seen by the kernels.
struct Dims {
    int n0, n1, n2;   // cells
    int hn0;          // n0 / 2 (split levels)
    int half;         // n0*n1*n2 / 2 (split levels)
    int ncell;        // n0*n1*n2
    int split;        // 1: checkerboard-split layout, 0: natural
    int rz;           // coarsening ratio in z to the next level (1 in 2-D)
};

// Index of cell (i, j, k) of a level in its storage layout.
__host__ __device__ __forceinline__ int level_index(const Dims& d, int i, int j, int k) {
    if (d.split) return ((i + j + k) & 1) * d.half + (j + d.n1 * k) * d.hn0 + (i >> 1);
    return i + d.n0 * (j + d.n1 * k);
}

// Boundary description for the prolongation ghosts (per direction, low/high).
struct BcDesc {
    int lo[3];
    int hi[3];
};

template <typename T>
struct LevelArrays {
    T* phi = nullptr;      // solution / correction
    T* f = nullptr;        // right-hand side
    T* bx = nullptr;       // low-face coefficients / h^2
    T* by = nullptr;
    T* bz = nullptr;
    T* diag = nullptr;
    T* invdiag = nullptr;
};

struct Level {
    Dims d;
    double h[3];
    LevelArrays<double> a64;
    LevelArrays<float> a32;
    // Dirichlet wall planes (beta'/h^2 of the wall faces), [dir][side]; null when not Dirichlet
    double* wall[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    double* alpha = nullptr;   // Helmholtz term in the level layout for this call (null: 0)
    double* alpha_store = nullptr;
};

// Reduction scratch (device) and its pinned host mirror.
struct Reduce {
    unsigned long long* maxbits = nullptr;  // running max of |r| as IEEE bits (non-negative)
    double* partial = nullptr;              // per-block partials (sum, max, min)
    double* scalars = nullptr;              // [0] mean, [1] fnorm, [2] sum, [3] max, [4] min
    int* counters = nullptr;                // [0] bottom iterations
    unsigned long long* h_maxbits = nullptr;
    double* h_scalars = nullptr;
    int* h_counters = nullptr;
    int nblocks_partial = 0;
};

struct BoxDesc {   // one fab of the caller's layout (device copy of the table)
    const double* ptr;
    int lo[3];
    int hi[3];
    int ext[3];    // fab extents incl. ghosts (and the +1 face along the edge direction)
    int ng;
    int comp_off;  // offset of the component inside the fab, in elements
};

}  // namespace mac

struct mac_ctx {
    mac_geom g{};
    mac_opts o{};
    std::vector<int> box_lo, box_hi;
    int dm = 3;
    int n[3] = {1, 1, 1};        // internal 3-D cell counts (2-D: n[2] = 1)
    int va = 2;                  // vertical direction index in the internal layout
    int bc_lo[3], bc_hi[3];
    double dx[3];
    bool singular = true;        // alpha == 0 and no Dirichlet face (this call)
    bool geom_singular = true;   // no Dirichlet face
    int nlevels = 1;
    std::vector<mac::Level> lev;
    cudaStream_t stream = nullptr;
    bool own_stream = false;     // created here because the caller passed none

    // fine-level inputs in natural layout (device)
    double* u[3] = {nullptr, nullptr, nullptr};   // faces (n_d + 1 along d)
    double* rho = nullptr;
    double* rhs = nullptr;
    double* phin = nullptr;                       // phi natural
    double* beta0 = nullptr;                      // [nr]
    double* beta0e = nullptr;                     // [nr+1]
    double* scratch = nullptr;                    // generic FP64 scratch (ncell)
    // caller-layout staging
    double* staging = nullptr;
    size_t staging_elems = 0;
    mac::BoxDesc* d_boxes = nullptr;
    mac::BoxDesc* h_boxes = nullptr;              // pinned
    int box_table_cap = 0;

    // bottom solver scratch
    double* bottom_scratch = nullptr;

    mac::Reduce red;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};

    // CUDA graphs of one V-cycle (fp64 and fp32 inner) and their kernel-node counts
    cudaGraphExec_t vc_exec[2] = {nullptr, nullptr};
    long long graph_kernels[2] = {0, 0};
    long long issued = 0;                         // kernels launched (host count)
    cudaEvent_t tev[8] = {};                      // per-iteration timing events (opts.timing)
    double ktime_ms[8] = {};
    int ktime_launches[8] = {};

    size_t bytes_allocated = 0;
    std::vector<void*> allocations;
};

namespace mac {

// ---- kernels / launchers (mac_kernels.cu) -------------------------------------------------
template <typename T>
void launch_gsrb(const Dims& d, int colour, LevelArrays<T>& a, cudaStream_t s);
template <typename T>
void launch_resid_restrict(const Dims& fine, const Dims& coarse, const LevelArrays<T>& a,
                           T* fc, bool red_only, cudaStream_t s);
template <typename T>
void launch_prolong_add(const Dims& fine, const Dims& coarse, const BcDesc& bc, const T* ec,
                        T* phi_fine, cudaStream_t s);
template <typename T>
void launch_resid_norm(const Dims& d, const LevelArrays<T>& a, bool red_only,
                       unsigned long long* maxbits, cudaStream_t s);
void launch_resid64_to32(const Dims& d, const LevelArrays<double>& a, float* r32,
                         unsigned long long* maxbits, cudaStream_t s);
void launch_accumulate(const Dims& d, double* phi, const float* e, cudaStream_t s);
template <typename Tio>
void launch_bottom(const Dims& d, const LevelArrays<double>& a64, Tio* x, const Tio* f,
                   double* scratch, bool singular, int nub, double eps, int max_iter,
                   int* iter_counter, cudaStream_t s);

// ---- setup kernels (mac_setup.cu) -----------------------------------------------------------
int setup_fine_coefficients(mac_ctx* c, const double* beta0, const double* beta0e);
int setup_coarse_levels(mac_ctx* c);
int setup_fp32_copies(mac_ctx* c);
int setup_rhs(mac_ctx* c, const double* macrhs, bool have_beta0);
int finish_rhs_stats(mac_ctx* c, double* fnorm_out, bool* finite_out);
int correct_velocity(mac_ctx* c, bool have_beta0);
int setup_fine_from_faces(mac_ctx* c, const double* fx, const double* fy, const double* fz,
                          const double* alpha_nat);
int setup_rhs_from(mac_ctx* c, const double* rh_nat);
int natural_to_level0(mac_ctx* c, const double* src, double* dst);
int level0_to_natural(mac_ctx* c, const double* src, double* dst);
int check_density(mac_ctx* c, bool* ok);

// caller box layout
int gather_cells(mac_ctx* c, int ptr_kind, const double* const* fabs, int ng, int ncomp, int comp,
                 double* dst);
int gather_faces(mac_ctx* c, int ptr_kind, const double* const* fabs, int ng, int dir,
                 double* dst);
int scatter_cells(mac_ctx* c, int ptr_kind, double* const* fabs, int ng, const double* src);
int scatter_faces(mac_ctx* c, int ptr_kind, double* const* fabs, int ng, int dir,
                  const double* src);

// ---- solver (mac_solver.cu) -----------------------------------------------------------------
int run_solve(mac_ctx* c, mac_stats* st);
// Forward projection on the whole-domain arrays already in c->u / c->rho / c->phin; leaves the
// level-0 coefficients and phi (level-0 layout) in place.
int forward_projection(mac_ctx* c, const double* macrhs, bool have_beta0, mac_stats* st);
int set_call_state(mac_ctx* c, bool with_alpha);
int load_beta0(mac_ctx* c, int ptr_kind, const double* b0, const double* b0e);
void begin_call_stats(mac_ctx* c, mac_stats* st);
void end_call_stats(mac_ctx* c, mac_stats* st);
int alloc_device(mac_ctx* c, void** p, size_t bytes);

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace mac
