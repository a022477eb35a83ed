// Allocation-free elliptic solve on a small single-box level.
//
// Who needs it: callers that must not allocate device memory -- a host code that hands all of
// the GPU's memory to its own pool allocator, a time-step loop that runs under a fixed memory
// budget, or code that calls in from a place where cudaMalloc is forbidden or too slow.  This
// entry point takes the caller's input and output arrays and keeps its own working storage in
// one fixed array compiled into the library, so nothing is allocated per call.
//
// It is the allocation-free variant of the single-CTA BiCGStab solver that the multigrid uses on
// its coarsest level (k_bottom in mac_kernels.cu): the same operator, the same Jacobi-
// preconditioned BiCGStab, here run to the caller's relative tolerance on the whole level.
//
// Limits and sharing rules:
//   * at most MAC_NOALLOC_MAX_CELLS cells; larger levels are rejected with MAC_ERR_TOO_LARGE;
//   * the working array (14 * MAC_NOALLOC_MAX_CELLS doubles, 459 KB) exists once per GPU that
//     loads the library and stays allocated until the process exits;
//   * every call uses the same array and leaves its contents behind; the kernels clear or
//     overwrite everything they read before reading it;
//   * calls that overlap on the GPU (different streams, or different host threads) race on the
//     array -- serialise them (one stream does that);
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress while that device is current.
//   * every max-norm propagates NaN (a NaN input makes the call return MAC_ERR_NONFINITE, never a
//     converged status).
#include <cmath>
#include <cstring>
#include <mutex>

#include "mac_internal.cuh"

namespace {

constexpr int kCells = MAC_NOALLOC_MAX_CELLS;
constexpr int kOpWords = 5;       // beta'_x, beta'_y, beta'_z, diag, 1/diag
constexpr int kVecWords = 9;      // x, f, r, r^, p, v, s, t, y
constexpr int kResultWords = 8;   // [0] true |r|/|f|, [1] iterations, [2] |f|, [3] status
constexpr int kThreads = 1024;
constexpr int kMaxDevices = 64;

// The only storage this entry point uses on the device (every GPU that loads the library keeps
// one copy until exit).
static __device__ __align__(256) double g_noalloc_scratch[(kOpWords + kVecWords) * kCells + kResultWords];

std::mutex g_mutex;
double* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once per device).
int scratch_address(double** out) {
    int dev = 0;
    MAC_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return MAC_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        MAC_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return MAC_OK;
}

struct NaGeom {
    int n[3];
    int active[3];
    int bc_lo[3], bc_hi[3];
    double ih2[3];
    int N;
};

// Operator of the level in natural layout: low-face beta' (0 on non-periodic walls), diagonal
// with Dirichlet walls (2 beta'_wall) and alpha, and its reciprocal.
__global__ void __launch_bounds__(256)
k_na_operator(NaGeom G, const double* __restrict__ fx, const double* __restrict__ fy,
              const double* __restrict__ fz, const double* __restrict__ alpha,
              double* __restrict__ op) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= G.N) return;
    const int i = q % G.n[0];
    const int row = q / G.n[0];
    const int j = row % G.n[1];
    const int k = row / G.n[1];
    const int c[3] = {i, j, k};
    const double* fin[3] = {fx, fy, fz};
    double diag = alpha ? alpha[q] : 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double lo_arm = 0.0;
        if (G.active[d]) {
            const int m0 = G.n[0] + (d == 0), m1 = G.n[1] + (d == 1);
            const int flo = i + m0 * (j + m1 * k);
            const int stride = d == 0 ? 1 : d == 1 ? m0 : m0 * m1;
            const double blo = fin[d][flo] * G.ih2[d];
            const double bhi = fin[d][flo + stride] * G.ih2[d];
            const bool per = G.bc_lo[d] == MAC_BC_PER;
            if (c[d] > 0 || per) {
                lo_arm = blo;
                diag += blo;
            } else if (G.bc_lo[d] == MAC_BC_DIR) {
                diag += 2.0 * blo;
            }
            if (c[d] < G.n[d] - 1 || per) diag += bhi;
            else if (G.bc_hi[d] == MAC_BC_DIR) diag += 2.0 * bhi;
        }
        op[d * G.N + q] = lo_arm;
    }
    op[3 * G.N + q] = diag;
    op[4 * G.N + q] = 1.0 / diag;
}

struct View {
    int n0, n1, n2, N;
    const double *bx, *by, *bz, *dg, *idg;
};

__device__ __forceinline__ double arms(const View& v, const double* __restrict__ x, int c) {
    const int i = c % v.n0;
    const int row = c / v.n0;
    const int j = row % v.n1;
    const int k = row / v.n1;
    const int ip = i == v.n0 - 1 ? 0 : i + 1, im = i == 0 ? v.n0 - 1 : i - 1;
    const int jp = j == v.n1 - 1 ? 0 : j + 1, jm = j == 0 ? v.n1 - 1 : j - 1;
    const int kp = k == v.n2 - 1 ? 0 : k + 1, km = k == 0 ? v.n2 - 1 : k - 1;
    const int cxp = ip + v.n0 * (j + v.n1 * k), cxm = im + v.n0 * (j + v.n1 * k);
    const int cyp = i + v.n0 * (jp + v.n1 * k), cym = i + v.n0 * (jm + v.n1 * k);
    const int czp = i + v.n0 * (j + v.n1 * kp), czm = i + v.n0 * (j + v.n1 * km);
    double s = v.bx[c] * x[cxm];
    s = fma(v.bx[cxp], x[cxp], s);
    s = fma(v.by[c], x[cym], s);
    s = fma(v.by[cyp], x[cyp], s);
    s = fma(v.bz[c], x[czm], s);
    s = fma(v.bz[czp], x[czp], s);
    return s;
}

__device__ double cta_sum(double v, double* sm) {
    const int t = threadIdx.x;
    sm[t] = v;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (t < o) sm[t] += sm[t + o];
        __syncthreads();
    }
    const double r = sm[0];
    __syncthreads();
    return r;
}

// max that keeps a NaN from either side (the library's fmax drops NaN and would hide a
// non-finite input)
__device__ __forceinline__ double nan_max(double acc, double v) {
    return (v > acc || v != v) ? v : acc;
}

__device__ double cta_max(double v, double* sm) {
    const int t = threadIdx.x;
    sm[t] = v;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (t < o) sm[t] = nan_max(sm[t], sm[t + o]);
        __syncthreads();
    }
    const double r = sm[0];
    __syncthreads();
    return r;
}

__device__ void apply(const View& v, const double* x, double* y) {
    for (int c = threadIdx.x; c < v.N; c += kThreads) y[c] = v.dg[c] * x[c] - arms(v, x, c);
    __syncthreads();
}

// One CTA: BiCGStab (Jacobi right preconditioner) on the whole level to
// ||f - A x||_inf <= eps ||f||_inf, restarted from the current x when the true residual is still
// above the tolerance after the recursive one met it.  All nine work vectors are (re)written
// before they are read.  The problem is singular when no face is Dirichlet (geom_singular) and
// alpha is NULL or zero everywhere; the mean of rh is then removed.
__global__ void __launch_bounds__(kThreads)
k_na_solve(View v, double* __restrict__ phi, const double* __restrict__ rh,
           const double* __restrict__ alpha, double* __restrict__ vec,
           double* __restrict__ result, int geom_singular, double eps, int max_iter) {
    __shared__ double sm[kThreads];
    const int N = v.N;
    const int tid = threadIdx.x;
    double* x = vec;
    double* f = vec + N;
    double* r = vec + 2 * N;
    double* rh0 = vec + 3 * N;
    double* p = vec + 4 * N;
    double* vv = vec + 5 * N;
    double* s = vec + 6 * N;
    double* t = vec + 7 * N;
    double* y = vec + 8 * N;
    double loc = 0.0;
    for (int c = tid; c < N; c += kThreads) {
        x[c] = phi[c];
        f[c] = rh[c];
        loc += f[c];
    }
    const double mean = cta_sum(loc, sm) / N;
    bool singular = geom_singular != 0;
    if (singular && alpha) {
        loc = 0.0;
        for (int c = tid; c < N; c += kThreads) loc = nan_max(loc, fabs(alpha[c]));
        singular = cta_max(loc, sm) == 0.0;
    }
    loc = 0.0;
    for (int c = tid; c < N; c += kThreads) {
        if (singular) f[c] -= mean;
        loc = nan_max(loc, fabs(f[c]));
    }
    const double fnorm = cta_max(loc, sm);
    int iters = 0;
    double rel = 0.0;
    if (fnorm == 0.0 || !isfinite(fnorm)) {
        for (int c = tid; c < N; c += kThreads) x[c] = 0.0;
        __syncthreads();
        rel = isfinite(fnorm) ? 0.0 : NAN;
    } else {
        const double tol = eps * fnorm;
        while (iters < max_iter) {
            // true residual of the current iterate
            apply(v, x, t);
            loc = 0.0;
            for (int c = tid; c < N; c += kThreads) {
                r[c] = f[c] - t[c];
                rh0[c] = r[c];
                p[c] = 0.0;
                vv[c] = 0.0;
                loc = nan_max(loc, fabs(r[c]));
            }
            const double rn0 = cta_max(loc, sm);
            rel = rn0 / fnorm;
            if (!(rn0 > tol)) break;
            double rho_old = 1.0, alpha = 1.0, omega = 1.0;
            bool restart = false;
            while (iters < max_iter && !restart) {
                ++iters;
                loc = 0.0;
                for (int c = tid; c < N; c += kThreads) loc += rh0[c] * r[c];
                const double rho = cta_sum(loc, sm);
                if (rho == 0.0) break;
                const double beta = (rho / rho_old) * (alpha / omega);
                for (int c = tid; c < N; c += kThreads) {
                    p[c] = r[c] + beta * (p[c] - omega * vv[c]);
                    y[c] = p[c] * v.idg[c];
                }
                __syncthreads();
                apply(v, y, vv);
                loc = 0.0;
                for (int c = tid; c < N; c += kThreads) loc += rh0[c] * vv[c];
                const double rv = cta_sum(loc, sm);
                if (rv == 0.0) break;
                alpha = rho / rv;
                for (int c = tid; c < N; c += kThreads) {
                    x[c] += alpha * y[c];
                    s[c] = r[c] - alpha * vv[c];
                    y[c] = s[c] * v.idg[c];
                }
                __syncthreads();
                apply(v, y, t);
                double l1 = 0.0, l2 = 0.0;
                for (int c = tid; c < N; c += kThreads) {
                    l1 += t[c] * s[c];
                    l2 += t[c] * t[c];
                }
                const double ts = cta_sum(l1, sm);
                const double tt = cta_sum(l2, sm);
                omega = tt > 0.0 ? ts / tt : 0.0;
                loc = 0.0;
                for (int c = tid; c < N; c += kThreads) {
                    x[c] += omega * y[c];
                    r[c] = s[c] - omega * t[c];
                    loc = nan_max(loc, fabs(r[c]));
                }
                const double rn = cta_max(loc, sm);
                if (!(rn > 0.5 * tol) || omega == 0.0) restart = true;
                rho_old = rho;
            }
            if (!restart) break;   // breakdown or iteration limit: report the true residual below
        }
        // final true residual
        apply(v, x, t);
        loc = 0.0;
        for (int c = tid; c < N; c += kThreads) loc = nan_max(loc, fabs(f[c] - t[c]));
        rel = cta_max(loc, sm) / fnorm;
    }
    for (int c = tid; c < N; c += kThreads) phi[c] = x[c];
    if (tid == 0) {
        result[0] = rel;
        result[1] = (double)iters;
        result[2] = fnorm;
    }
}

}  // namespace

extern "C" int mac_solve_small_noalloc(int dm, const int* n, const double* dx, const int* bc_lo,
                                       const int* bc_hi, const double* rh, double* phi,
                                       const double* beta_x, const double* beta_y,
                                       const double* beta_z, const double* alpha, double rel_eps,
                                       int max_iter, void* cuda_stream, mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if ((dm != 2 && dm != 3) || !n || !dx || !bc_lo || !bc_hi || !rh || !phi || !beta_x ||
        !beta_y || (dm == 3 && !beta_z) || max_iter < 0 || !(rel_eps > 0.0))
        return st->status = MAC_ERR_INVALID;
    NaGeom G;
    long long N = 1;
    bool has_dir = false;
    for (int d = 0; d < 3; ++d) {
        const bool act = d < dm;
        G.n[d] = act ? n[d] : 1;
        G.active[d] = act ? 1 : 0;
        G.bc_lo[d] = act ? bc_lo[d] : MAC_BC_NEU;
        G.bc_hi[d] = act ? bc_hi[d] : MAC_BC_NEU;
        if (act) {
            if (n[d] < 1 || !(dx[d] > 0.0)) return st->status = MAC_ERR_INVALID;
            const int bl = bc_lo[d], bh = bc_hi[d];
            if ((bl != MAC_BC_PER && bl != MAC_BC_DIR && bl != MAC_BC_NEU) ||
                (bh != MAC_BC_PER && bh != MAC_BC_DIR && bh != MAC_BC_NEU) ||
                ((bl == MAC_BC_PER) != (bh == MAC_BC_PER)))
                return st->status = MAC_ERR_INVALID;
            has_dir = has_dir || bl == MAC_BC_DIR || bh == MAC_BC_DIR;
            G.ih2[d] = 1.0 / (dx[d] * dx[d]);
        } else {
            G.ih2[d] = 0.0;
        }
        N *= G.n[d];
    }
    if (N > kCells) return st->status = MAC_ERR_TOO_LARGE;
    G.N = (int)N;
    double* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return st->status = rc;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    double* op = scratch;
    double* vec = scratch + kOpWords * kCells;
    double* result = scratch + (kOpWords + kVecWords) * kCells;
    k_na_operator<<<(G.N + 255) / 256, 256, 0, s>>>(G, beta_x, beta_y, dm == 3 ? beta_z : nullptr,
                                                    alpha, op);
    MAC_CUDA_TRY(cudaGetLastError());
    View v;
    v.n0 = G.n[0];
    v.n1 = G.n[1];
    v.n2 = G.n[2];
    v.N = G.N;
    v.bx = op;
    v.by = op + G.N;
    v.bz = op + 2 * G.N;
    v.dg = op + 3 * G.N;
    v.idg = op + 4 * G.N;
    k_na_solve<<<1, kThreads, 0, s>>>(v, phi, rh, alpha, vec, result, has_dir ? 0 : 1, rel_eps,
                                      max_iter);
    MAC_CUDA_TRY(cudaGetLastError());
    double res[3] = {0.0, 0.0, 0.0};
    MAC_CUDA_TRY(cudaMemcpyAsync(res, result, sizeof(res), cudaMemcpyDeviceToHost, s));
    MAC_CUDA_TRY(cudaStreamSynchronize(s));
    st->rel_resid = res[0];
    st->vcycles = (int)res[1];
    st->fnorm = res[2];
    st->nlevels = 1;
    st->launches = 2;
    if (!std::isfinite(res[0]) || !std::isfinite(res[2])) return st->status = MAC_ERR_NONFINITE;
    return st->status = (res[0] <= rel_eps ? MAC_OK : MAC_ERR_NOT_CONVERGED);
}
