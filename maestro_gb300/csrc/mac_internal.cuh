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
#include <cstring>
#include <functional>
#include <utility>
#include <vector>

#include "maestro_mac.h"

namespace mac {

constexpr int kMaxLevels = 32;
constexpr int kBottomMaxCells = 65536;   // single-CTA bottom solver limit
constexpr int kBotScrPerCell = 18;       // bottom solver scratch: 14 doubles + 7 ints per cell

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

// 1/x in FP64 without the division instruction sequence: the hardware reciprocal estimate
// (rcp.approx.ftz.f64, on the special-function unit) refined by one third-order Newton step
// y <- y0 + y0 (e + e^2), e = 1 - x y0, which cubes the estimate's relative error, so the result
// is within rounding of 1/x.  Zero, subnormal, huge or non-finite inputs (tested on the exponent
// bits: no FP64 instruction) use the IEEE division.
__device__ __forceinline__ double recip_nr(double x) {
    const unsigned ex = (unsigned)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7FFu;
    if (ex < 64u || ex > 1980u) return 1.0 / x;
    double y0;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y0) : "d"(x));
    const double e = fma(-x, y0, 1.0);
    return fma(y0, fma(e, e, e), y0);
}

// FP64 <-> FP32 conversions on the integer pipe.  On GB300 a conversion instruction between FP64
// and FP32 occupies the scarce FP64 pipe like an FMA; in the FP64-bound kernels (the refinement
// residual, the accumulation, the coefficient setup) these bit-level versions keep it free.
// Results equal the hardware conversions (round to nearest even); operands outside the normal
// FP32 range (zero excepted), infinities and NaNs take the hardware path.
__device__ __forceinline__ float to_float_rn(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(u >> 52) & 0x7FFu;
    if (e >= 897u && e <= 1150u) {   // normal FP32 exponents 1 .. 254
        const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
        const unsigned rem = (unsigned)(m & 0x1FFFFFFFull);   // the 29 dropped bits
        unsigned r = ((unsigned)(u >> 63) << 31) | ((e - 896u) << 23) | (unsigned)(m >> 29);
        r += (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ? 1u : 0u;
        return __uint_as_float(r);
    }
    return __double2float_rn(x);
}
__device__ __forceinline__ double to_double(float f) {
    const unsigned v = __float_as_uint(f);
    const unsigned e = (v >> 23) & 0xFFu;
    if (e - 1u < 254u) {   // normal
        const unsigned long long d = ((unsigned long long)(v >> 31) << 63) |
                                     ((unsigned long long)(e + 896u) << 52) |
                                     ((unsigned long long)(v & 0x7FFFFFu) << 29);
        return __longlong_as_double((long long)d);
    }
    if ((v & 0x7FFFFFFFu) == 0u) return __longlong_as_double((long long)((unsigned long long)(v >> 31) << 63));
    return (double)f;
}

// Order-preserving map of a double onto unsigned 64-bit integers (max/min on the integer pipe;
// NaN maps above +inf / below -inf depending on its sign bit).
__device__ __forceinline__ unsigned long long ordered_bits(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
__host__ __device__ inline double from_ordered_bits(unsigned long long u) {
    const unsigned long long b = (u >> 63) ? (u & 0x7FFFFFFFFFFFFFFFULL) : ~u;
    double d;
    memcpy(&d, &b, sizeof(d));
    return d;
}

// Positive, finite double (integer test on the bit pattern: no FP64 instructions).
__device__ __forceinline__ bool positive_finite(double v) {
    const long long b = __double_as_longlong(v);
    return b > 0 && b < 0x7FF0000000000000LL;
}

// Per-layer factor tables (k_beta0_tables), nr+1 entries each, vertical index r:
enum {
    kTabFac0 = 0,   // beta0_f^p * 2 / h_d^2 of the low face along d (3 tables: d = 0, 1, 2)
    kTabG0 = 3,     // beta0_f / dx_d (3 tables): divergence of beta0 U
    kTabK0 = 6,     // h_d / beta0_f (3 tables): correction U -= beta' K (phi_hi - phi_lo)
    kTabCount = 9
};

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
    double* scalars = nullptr;              // [0] mean, [1] fnorm, [2] sum, [3] max, [4] min,
                                            // [5] OR of the guess's bits (0: phi = +0)
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

// Finest-level FP32 kernels with face coefficients computed from rho32 (mixed precision).
// Per-layer FP32 face factors beta0_f^p * 2 / h_d^2 (tables of nr+1 floats, vertical index r):
//   0: x faces; 1: y faces (3-D: horizontal; 2-D: unused); 2: low vertical face of layer r,
//   3: high vertical face of layer r -- both zero where the face is a non-periodic wall;
//   4: Dirichlet diagonal term of layer r (wall factor of the vertical walls touching it).
constexpr int kOtfTables = 5;
struct OtfParams {
    int n[3];
    int per[3];
    int dlo[3], dhi[3];   // Dirichlet flags
    int has_dir;          // any Dirichlet face
    int va;
    int dm;
    const float* fac;     // kOtfTables tables of (n[va] + 1)
    const float* rho;     // level-0 layout
    // staged 3-D half-sweep (rows of whole colour-half planes copied to shared memory by bulk
    // async copies); ty == 0: not applicable, the per-cell kernel runs instead
    int ty;               // rows of a tile
    int zc, nz;           // planes per block, blocks along z
    int smem;             // dynamic shared memory bytes
    int rty, rzc, rnz, rsmem;   // the same for the staged defect + restriction (rty == 0: none)
    int* err;             // device flag: a bounded wait on a copy gave up
    float omega;          // relaxation weight of the half-sweeps (1: Gauss-Seidel)
    unsigned long long wait_ns;   // limit of a wait for the block's own copies (ns)
    int inject_expiry;    // test: the first wait targets a barrier no copy completes
    // fused red + black sweep (fty == 0: not applicable, the half-sweeps run instead)
    int fty;              // rows of a tile
    int fzc, fnz;         // planes per block, blocks along z
    int fst;              // shared-memory ring stages
    int fsmem;            // dynamic shared memory bytes
    int fthreads;         // threads per block: (fty + 2) rows x hn0 / 4
};
// Tile plan of the staged half-sweep for the finest level (OtfParams.ty/zc/nz/smem).
void plan_otf_tile(const Dims& d, int dm, int sms, OtfParams& P);

// Flexible-CG vectors of the mixed-precision inner solve (level-0 layout, FP32): search
// direction p, q = L p, accumulated correction x, the colour-0 half of w = L z; the inner-product
// partials, [0] alpha [1] beta [2] (p, q) of the last step, and the finished-block counter.
struct KrylovBufs {
    float* p = nullptr;
    float* q = nullptr;
    float* x = nullptr;
    float* w0 = nullptr;
    double* partial = nullptr;
    double* scalars = nullptr;
    unsigned* count = nullptr;
};

struct AmrState;   // multi-level (AMR) hierarchy of a context (mac_amr.cu)
struct HgState;    // nodal (HG) projection hierarchy of a context (hg_nodal.cu)

}  // namespace mac

constexpr int kInnerGraphs = 8;   // mixed-precision steps of up to 8 inner V-cycles are graphed

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
    // per vertical index r: the kTab* factor tables, (nr+1) doubles each
    double* b0tab = nullptr;
    double* scratch = nullptr;                    // generic FP64 scratch (ncell)
    double* base1d = nullptr;                     // 4 x (nr + 1) base-state values
    // caller-layout staging (host-pointer calls): one region per array of a call, filled and
    // drained by the copy engines on the transfer stream
    double* staging = nullptr;
    size_t staging_elems = 0;
    size_t staging_cursor = 0;
    cudaStream_t xfer = nullptr;               // host <-> device copies of host-pointer calls
    cudaEvent_t xev[16] = {};                  // cross-stream ordering events (ring)
    int xev_next = 0;
    mac::BoxDesc* d_boxes = nullptr;
    mac::BoxDesc* h_boxes = nullptr;              // pinned
    int box_table_cap = 0;

    // bottom solver scratch
    double* bottom_scratch = nullptr;

    mac::Reduce red;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};

    // CUDA graphs of one outer iteration and their kernel-node counts: slot 0 the FP64 V-cycle,
    // slot v (1..kInnerGraphs) a mixed-precision step with v inner FP32 V-cycles
    cudaGraphExec_t vc_exec[kInnerGraphs + 1] = {};
    long long graph_kernels[kInnerGraphs + 1] = {};
    int cur_inner = 1;   // inner V-cycles of the next mixed-precision refinement step
    int sms = 0;         // SM count of the device
    mac::OtfParams otf_tile;  // tile plan of the staged finest-level half-sweep (ty/zc/nz/smem)
    long long issued = 0;                         // kernels launched (host count)
    cudaEvent_t tev[4][8] = {};                   // timing events of up to 4 V-cycles per iteration
    cudaEvent_t tail[3] = {};                     // before/after accumulation, after the residual
    int vtimer = 0;                               // inner V-cycle being issued (timing slot)
    // finest level of the mixed solve: FP32 density (level-0 layout) and the per-layer FP32 face
    // factors of OtfParams (kOtfTables tables of nr+1), for coefficients computed on the fly
    float* rho32 = nullptr;
    float* fac32 = nullptr;
    bool otf = false;                             // finest-level FP32 kernels use rho32
    mac::KrylovBufs kry;                          // flexible-CG vectors (allocated on first use)
    bool mean_pending = false;                    // f still holds the mean (singular problem)
    float* def_b = nullptr;                       // colour-1 defects of the finest FP32 level
    float* e_alt = nullptr;                       // second finest FP32 correction (fused sweeps)
    // spherical form (beta0 on every face): solver beta and beta0 face arrays (lazily allocated)
    double* cbeta[3] = {nullptr, nullptr, nullptr};
    double* cb0[3] = {nullptr, nullptr, nullptr};
    double* bot_inv = nullptr;                    // dense bottom (pseudo-)inverse (small bottoms)
    cudaStream_t aux = nullptr;                   // side stream of the bottom inverse
    cudaEvent_t aux_ev[2] = {nullptr, nullptr};   // [0] operators ready, [1] inverse done
    bool inv_pending = false;                     // the main stream still has to wait on aux_ev[1]
    int tail_start[2] = {-1, -1};                 // first tail level (FP64, FP32); -1: none
    size_t tail_smem[2] = {0, 0};
    double ktime_ms[8] = {};
    int ktime_launches[8] = {};

    mac::AmrState* amr = nullptr;                 // finer AMR levels (mac_ctx_set_amr); null: one level
    mac::HgState* hgs = nullptr;                  // nodal projection levels (first nodal call)
    int inflow_lo[3] = {0, 0, 0};                 // nodal projection: inflow (inlet) faces
    int inflow_hi[3] = {0, 0, 0};

    size_t bytes_allocated = 0;
    std::vector<void*> allocations;
};

namespace mac {

// ---- kernels / launchers (mac_kernels.cu) -------------------------------------------------
// omega != 1: over-relaxed update e = e_old + omega (e_GS - e_old)
template <typename T>
void launch_gsrb(const Dims& d, int colour, LevelArrays<T>& a, cudaStream_t s, T omega = T(1));
template <typename T>
void launch_resid_restrict(const Dims& fine, const Dims& coarse, const LevelArrays<T>& a,
                           T* fc, T* ec, bool red_only, cudaStream_t s);
// phi_in (optional): read the fine values from phi_in instead of phi_fine (out of place; the
// cells the kernel does not update keep phi_fine's values)
template <typename T>
void launch_prolong_add(const Dims& fine, const Dims& coarse, const BcDesc& bc, const T* ec,
                        T* phi_fine, bool black_only, cudaStream_t s, const T* phi_in = nullptr);
template <typename T>
void launch_resid_norm(const Dims& d, const LevelArrays<T>& a, bool red_only,
                       unsigned long long* maxbits, cudaStream_t s);
// r32 = f - L phi (FP64 arithmetic, FP32 result) and its max-norm; e32 (optional) is zeroed in
// the same pass (the next inner solve starts from e = 0)
void launch_resid64_to32(const Dims& d, const LevelArrays<double>& a, float* r32,
                         unsigned long long* maxbits, cudaStream_t s, float* e32 = nullptr);
// the initial residual of a zero guess: f -= mean (mean non-null), r32 = f, e32 = 0, max |f|
void launch_first_resid_zero(const Dims& d, double* f, const double* mean, float* r32,
                             float* e32, unsigned long long* maxbits, cudaStream_t s);
void launch_accumulate(const Dims& d, double* phi, const float* e, cudaStream_t s);

// flexible CG around the FP32 V-cycle (mac_krylov.cu); A.phi = z (the V-cycle output), A.f = r
int krylov_partials(const Dims& d);
void launch_fcg_dots(const Dims& d, int dm, bool otf, const OtfParams& P,
                     const LevelArrays<float>& A, const KrylovBufs& K, bool first, bool store_w,
                     cudaStream_t s);
void launch_fcg_update(const Dims& d, const LevelArrays<float>& A, const KrylovBufs& K,
                       bool first, cudaStream_t s);
void launch_fcg_final(const Dims& d, double* phi, const LevelArrays<float>& A,
                      const KrylovBufs& K, bool first, cudaStream_t s);

// dout (optional, over-relaxed staged half-sweeps only): the updated cells' defects f - L e,
// colour-half indexing; launch_gsrb_otf returns without writing it where it does not apply
void launch_gsrb_otf(const Dims& d, const OtfParams& P, int colour, float* e, const float* r,
                     cudaStream_t s, float* dout = nullptr);
// blk (optional): colour-1 defects written by the preceding over-relaxed colour-1 half-sweep;
// with red_only false the staged kernel then forms only the colour-0 defects and adds them
void launch_resid_restrict_otf(const Dims& fine, const Dims& coarse, const OtfParams& P,
                               const float* e, const float* r, float* fc, float* ec,
                               bool red_only, cudaStream_t s, const float* blk = nullptr);
// whether the staged half-sweep and defect kernels run on this level (then dout/blk apply)
inline bool otf_staged(const OtfParams& P) { return P.dm == 3 && P.ty > 0 && P.rty > 0; }
// one whole red/black sweep of the finest FP32 level, ein -> eout (both colours; ein != eout);
// dout (optional): the colour-1 defects after the sweep, as launch_gsrb_otf's colour-1 dout
void launch_sweep_otf_fused(const Dims& d, const OtfParams& P, const float* ein, float* eout,
                            const float* r, cudaStream_t s, float* dout = nullptr);


template <typename Tio>
void launch_bottom(const Dims& d, const LevelArrays<double>& a64, Tio* x, const Tio* f,
                   double* scratch, bool singular, int nub, double eps, int max_iter,
                   int* iter_counter, cudaStream_t s);

int prepare_kernels();

// ---- single-CTA tail V-cycle (mac_tail.cu) --------------------------------------------------
constexpr int kTailMaxLevels = 8;
constexpr int kTailSmemMax = 200 * 1024;
template <typename T>
struct TailParams {
    int nlev;                             // tail levels above the bottom
    Dims lev[kTailMaxLevels];             // their dimensions (checkerboard-split in global memory)
    const T* bx[kTailMaxLevels];
    const T* by[kTailMaxLevels];
    const T* bz[kTailMaxLevels];
    const T* dg[kTailMaxLevels];
    const T* idg[kTailMaxLevels];
    Dims bottom;                          // bottom level (natural layout, FP64 operator)
    const double *bbx, *bby, *bbz, *bdg, *bidg;
    const T* f0;                          // right-hand side of the first tail level
    T* e0;                                // its correction (output)
    BcDesc bc;
    int nu1, nu2, nub, singular, bottom_max_iter;
    double bottom_eps;
    int* iters;
    const double* binv;                   // dense (pseudo-)inverse of the bottom; null: BiCGStab
    T omega;                              // relaxation weight of the half-sweeps (1: Gauss-Seidel)
};
template <typename T>
size_t tail_smem_bytes(const Dims* lev, int nl, const Dims& bottom);
template <typename T>
void launch_tail(const TailParams<T>& P, size_t smem, cudaStream_t s);
int prepare_tail_kernels();
// exact bottom solve of the FP32 V-cycle: bottoms of at most kDenseBottomMax cells, row r of the
// inverse applied by kDenseSeg lanes of a warp
constexpr int kDenseBottomMax = 64;
constexpr int kDenseSeg = 16;
void launch_bottom_inverse(const Dims& d, const double* bx, const double* by, const double* bz,
                           const double* dg, bool singular, double* out, cudaStream_t s);

// ---- setup kernels (mac_setup.cu) -----------------------------------------------------------
int setup_fine_coefficients(mac_ctx* c, const double* beta0, const double* beta0e);
int setup_coarse_levels(mac_ctx* c);
// the exact bottom's (pseudo-)inverse, on the side stream once the bottom operator is built
// (no-op unless the FP32 V-cycle uses it); run_solve orders the V-cycles after it
int issue_bottom_inverse(mac_ctx* c);
int setup_fp32_copies(mac_ctx* c);
// phi_nat (optional): the initial guess in natural layout, moved into the level-0 phi in the same pass
int setup_rhs(mac_ctx* c, const double* macrhs, bool have_beta0, const double* phi_nat = nullptr);
int finish_rhs_stats(mac_ctx* c, double* fnorm_out, bool* finite_out);
// f -= mean on level 0 (red.scalars[0]); the solve issues it for singular problems
void launch_sub_mean(mac_ctx* c);
// after_dir (optional) runs after the direction's correction kernel is queued (host-pointer
// calls start that direction's copy-back there); phi_nat_out (optional) receives phi in natural
// layout from the x-direction pass.
int correct_velocity(mac_ctx* c, bool have_beta0,
                     const std::function<int(int)>* after_dir = nullptr,
                     double* phi_nat_out = nullptr);
// reset_flags: clear the device flags (bad density, ...) first; false when a kernel of the same
// setup already raised one
int setup_fine_from_faces(mac_ctx* c, const double* fx, const double* fy, const double* fz,
                          const double* alpha_nat, bool reset_flags = true);
int setup_rhs_from(mac_ctx* c, const double* rh_nat, const double* phi_nat = nullptr);
int natural_to_level0(mac_ctx* c, const double* src, double* dst);
int level0_to_natural(mac_ctx* c, const double* src, double* dst);
int natural_to_level0(mac_ctx* c, const float* src, float* dst);
int level0_to_natural(mac_ctx* c, const float* src, float* dst);
int check_density(mac_ctx* c, bool* ok);

// caller box layout
// Gather split in two: gather_begin issues the host -> device copies of the fabs (transfer
// stream, host pointers only); gather_end orders the main stream after them and launches the
// gather kernel.  Work that does not need the array can be issued in between.
struct PendingGather {
    int ptr_kind = 0, ng = 0, ncomp = 1, comp = 0, dir = -1;
    const double* const* fabs = nullptr;
    double* dst = nullptr;
    double* region = nullptr;   // staging region (host pointers)
    cudaEvent_t ev = nullptr;
};
int staging_reserve(mac_ctx* c, size_t total_elems);
size_t host_fab_elems(const mac_ctx* c, int dir, int ng);
int gather_begin(mac_ctx* c, int ptr_kind, const double* const* fabs, int ng, int ncomp, int comp,
                 int dir, double* dst, PendingGather* pg);
int gather_end(mac_ctx* c, const PendingGather& pg);
int gather_cells(mac_ctx* c, int ptr_kind, const double* const* fabs, int ng, int ncomp, int comp,
                 double* dst);
int gather_faces(mac_ctx* c, int ptr_kind, const double* const* fabs, int ng, int dir,
                 double* dst);
int scatter_cells(mac_ctx* c, int ptr_kind, double* const* fabs, int ng, const double* src);
int scatter_faces(mac_ctx* c, int ptr_kind, double* const* fabs, int ng, int dir,
                  const double* src);

// ---- solver (mac_solver.cu) -----------------------------------------------------------------
int run_solve(mac_ctx* c, mac_stats* st);
// One FP64 V-cycle of the level-0 multigrid on (lev[0].a64.phi, lev[0].a64.f), in place.
int level0_fp64_vcycle(mac_ctx* c);
// One FP32 V-cycle (the mixed-precision inner cycle) on (lev[0].a32.phi, lev[0].a32.f), in
// place; the FP32 operator copies must be set up (setup_fp32_copies).
int level0_fp32_vcycle(mac_ctx* c);

// ---- multi-level hierarchy (mac_amr.cu) -------------------------------------------------------
// Validate and store the finer levels' boxes (levels 1 .. nlev-1) and allocate their arrays.
int amr_configure(mac_ctx* c, int nlev, const int* nboxes, const int* box_lo, const int* box_hi);
void amr_release(mac_ctx* c);
// ---- nodal projection (hg_nodal.cu) -----------------------------------------------------------
void hg_release(mac_ctx* c);
// Forward projection on the whole-domain arrays already in c->u / c->rho / c->phin; leaves the
// level-0 coefficients and phi (level-0 layout) in place.
int forward_projection(mac_ctx* c, const double* macrhs, bool have_beta0, mac_stats* st);
int set_call_state(mac_ctx* c, bool with_alpha);
// finest FP32 level with coefficients from rho on the fly (mixed MAC projection) or stored
int set_otf_mode(mac_ctx* c, bool on);
void report_call(const mac_ctx* c, const char* what, const mac_stats* st);
int load_beta0(mac_ctx* c, int ptr_kind, const double* b0, const double* b0e);
void begin_call_stats(mac_ctx* c, mac_stats* st);
void end_call_stats(mac_ctx* c, mac_stats* st);
int alloc_device(mac_ctx* c, void** p, size_t bytes);

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

// ---- kernel launch of the V-cycle chain ---------------------------------------------------------
// The kernels of one outer iteration form a chain on one stream.  They are launched with
// programmatic stream serialisation: a kernel's grid is scheduled while its predecessor drains.
// Every chain kernel starts with pdl_wait() (returns once the predecessor has completed and its
// writes are visible; no global access comes before it) followed by pdl_trigger() (lets the next
// kernel be scheduled).  Both are no-ops for a kernel launched without the attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
template <typename... KArgs, typename... Args>
inline void launch_chain(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                         cudaStream_t s, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// 3-D launch over an (nx, ny, nz) index space (x fastest): 128-thread blocks of (bx, 128/bx)
// with bx the smallest power of two >= nx, at most 128; z = blockIdx.z.  Kernels recover their
// indices without integer division.
struct Grid3 {
    dim3 grid, block;
};
inline Grid3 grid3(int nx, int ny, int nz) {
    int bx = 1;   // narrow rows share a warp (bx < 32), so no lane idles on small levels
    while (bx < nx && bx < 128) bx <<= 1;
    const int by = 128 / bx;
    Grid3 g;
    g.block = dim3(bx, by, 1);
    g.grid = dim3(ceil_div(nx, bx), ceil_div(ny, by), nz);
    return g;
}

// Launch grid of the right-hand-side kernel (each block covers kRhsPlanes planes); its block
// count sizes the partial-sum buffer.
constexpr int kRhsPlanes = 16;
constexpr int kRhsPartials = 4;   // per block: sum, max, min of f; OR of the guess's bits
inline Grid3 rhs_grid(const int* n) {
    Grid3 g = grid3(n[0], n[1], 1);
    g.grid.z = ceil_div(n[2], kRhsPlanes);
    return g;
}

}  // namespace mac
