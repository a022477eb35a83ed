// Context, V-cycle driver, mixed-precision refinement loop and the C ABI of the GB300 MAC
// projection.
//
// Solve structure (FBoxLib ml_cc as used by Source/mac_multigrid.f90:56-67, Docs/mg/mg.tex:325-375):
//   FP64  : repeat { V(nu1,nu2)-cycle on (phi, f); ||f - L phi||_inf } until
//           ||r|| <= rel_eps ||f|| (or abs_eps), at most max_vcycles times.
//   MIXED : r = f - L phi in FP64 (stored FP32); repeat { e = FP32 V-cycles on (e, r) from e = 0
//           (with an FP64 bottom solve), combined by flexible CG (inner_krylov) or applied one
//           after the other; phi += e in FP64; r = f - L phi in FP64 } until converged.
// Every V-cycle (with its convergence residual) is captured once into a CUDA graph and replayed;
// the host reads one 8-byte max-norm per cycle.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <functional>
#include <mutex>
#include <string>
#include <type_traits>

#include "mac_internal.cuh"

namespace mac {

namespace {
thread_local std::string g_last_cuda;

double bits_to_double(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
}

}  // namespace

void set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s: %s (%s:%d)", cudaGetErrorString(e), what, file, line);
    g_last_cuda = buf;
}

int alloc_device(mac_ctx* c, void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return MAC_OK;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return MAC_ERR_ALLOC;
    }
    c->allocations.push_back(*p);
    c->bytes_allocated += bytes;
    return MAC_OK;
}

namespace {

template <typename T>
int alloc_arr(mac_ctx* c, T** p, size_t n) {
    return alloc_device(c, reinterpret_cast<void**>(p), n * sizeof(T));
}

int alloc_level_fp32(mac_ctx* c, Level& L) {
    if (L.a32.bx) return MAC_OK;
    const size_t n = L.d.ncell;
    int rc = 0;
    rc |= alloc_arr(c, &L.a32.phi, n);
    rc |= alloc_arr(c, &L.a32.f, n);
    rc |= alloc_arr(c, &L.a32.bx, n);
    rc |= alloc_arr(c, &L.a32.by, n);
    rc |= alloc_arr(c, &L.a32.bz, n);
    rc |= alloc_arr(c, &L.a32.diag, n);
    rc |= alloc_arr(c, &L.a32.invdiag, n);
    return rc ? MAC_ERR_ALLOC : MAC_OK;
}

BcDesc bc_desc(const mac_ctx* c) {
    BcDesc b;
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = c->bc_lo[d];
        b.hi[d] = c->bc_hi[d];
    }
    return b;
}

// Host-side recursion issuing one V-cycle on levels l..L-1 (FP64 or FP32 arrays).
template <typename T>
LevelArrays<T>& arrays(Level& L);
template <>
LevelArrays<double>& arrays<double>(Level& L) { return L.a64; }
template <>
LevelArrays<float>& arrays<float>(Level& L) { return L.a32; }

OtfParams otf_params(const mac_ctx* c) {
    OtfParams P;
    for (int d = 0; d < 3; ++d) {
        P.n[d] = c->n[d];
        P.per[d] = (d < c->dm && c->bc_lo[d] == MAC_BC_PER) ? 1 : 0;
        P.dlo[d] = (d < c->dm && c->bc_lo[d] == MAC_BC_DIR) ? 1 : 0;
        P.dhi[d] = (d < c->dm && c->bc_hi[d] == MAC_BC_DIR) ? 1 : 0;
    }
    P.has_dir = 0;
    for (int d = 0; d < 3; ++d) P.has_dir |= P.dlo[d] | P.dhi[d];
    P.va = c->va;
    P.dm = c->dm;
    P.fac = c->fac32;
    P.rho = c->rho32;
    P.ty = c->otf_tile.ty;
    P.zc = c->otf_tile.zc;
    P.nz = c->otf_tile.nz;
    P.smem = c->otf_tile.smem;
    P.rty = c->otf_tile.rty;
    P.rzc = c->otf_tile.rzc;
    P.rnz = c->otf_tile.rnz;
    P.rsmem = c->otf_tile.rsmem;
    P.err = c->red.counters + 2;
    P.omega = (float)c->o.inner_omega;
    P.wait_ns = (unsigned long long)(c->o.wait_limit_s * 1e9);
    P.inject_expiry = c->o.inject_wait_expiry;
    P.fty = c->otf_tile.fty;
    P.fzc = c->otf_tile.fzc;
    P.fnz = c->otf_tile.fnz;
    P.fst = c->otf_tile.fst;
    P.fsmem = c->otf_tile.fsmem;
    P.fthreads = c->otf_tile.fthreads;
    return P;
}

inline void mark(mac_ctx* c, bool on, int slot) {
    if (on && c->vtimer < 4)
        cudaEventRecordWithFlags(c->tev[c->vtimer][slot], c->stream, cudaEventRecordExternal);
}

// Whole red/black sweeps of the finest FP32 level as one kernel each (ping-pong between a32.phi
// and e_alt; the V-cycle ends in a32.phi).
// The context's tile plans (otf_tile holds the plans only; its geometry fields are set per call
// by otf_params) admit the fused sweep on level 0.
bool fused_plan(const mac_ctx* c) {
    const OtfParams& T = c->otf_tile;
    return c->dm == 3 && T.ty > 0 && T.rty > 0 && T.fty > 0;
}
bool fused_sweeps(const mac_ctx* c) {
    return c->otf && c->o.fused_sweep && c->e_alt != nullptr && fused_plan(c);
}

// The FP32 V-cycle's bottom solved exactly by the dense (pseudo-)inverse (small bottoms, run
// through the tail kernel); the FP64 V-cycle keeps BiCGStab.
bool exact_bottom(const mac_ctx* c) {
    return c->o.inner_exact_bottom && c->o.coarse_tail && c->bot_inv != nullptr;
}

// GS-RB sweeps down / up a V-cycle: the FP32 (inner, mixed-precision) V-cycle may use its own
// counts (inner_nu1/inner_nu2 >= 0), the FP64 V-cycle always uses nu1/nu2.
int sweeps_down(const mac_ctx* c, bool fp32) {
    return fp32 && c->o.inner_nu1 >= 0 ? c->o.inner_nu1 : c->o.nu1;
}
int sweeps_up(const mac_ctx* c, bool fp32) {
    return fp32 && c->o.inner_nu2 >= 0 ? c->o.inner_nu2 : c->o.nu2;
}

template <typename T>
void vcycle(mac_ctx* c, int l) {
    Level& L = c->lev[l];
    LevelArrays<T>& a = arrays<T>(L);
    const mac_opts& o = c->o;
    const bool tm = o.timing && l == 0;
    const bool otf = std::is_same<T, float>::value && l == 0 && c->otf;
    const int nu1 = sweeps_down(c, std::is_same<T, float>::value);
    const int nu2 = sweeps_up(c, std::is_same<T, float>::value);
    // over-relaxation (FP32 V-cycle only); the red-only defect and the black-only prolongation
    // rest on plain Gauss-Seidel half-sweeps
    const T omega = std::is_same<T, float>::value ? T(c->o.inner_omega) : T(1);
    const bool gs = omega == T(1);
    if (l == c->nlevels - 1) {
        launch_bottom<T>(L.d, L.a64, a.phi, a.f, c->bottom_scratch, c->singular, o.nub,
                         o.bottom_eps, o.bottom_max_iter, c->red.counters, c->stream);
        ++c->issued;
        return;
    }
    const int tslot = std::is_same<T, float>::value ? 1 : 0;
    if (o.coarse_tail && l == c->tail_start[tslot]) {
        TailParams<T> tp;
        tp.nlev = c->nlevels - 1 - l;
        for (int q = 0; q < tp.nlev; ++q) {
            Level& Lq = c->lev[l + q];
            LevelArrays<T>& aq = arrays<T>(Lq);
            tp.lev[q] = Lq.d;
            tp.bx[q] = aq.bx;
            tp.by[q] = aq.by;
            tp.bz[q] = aq.bz;
            tp.dg[q] = aq.diag;
            tp.idg[q] = aq.invdiag;
        }
        Level& B = c->lev[c->nlevels - 1];
        tp.bottom = B.d;
        tp.bbx = B.a64.bx;
        tp.bby = B.a64.by;
        tp.bbz = B.a64.bz;
        tp.bdg = B.a64.diag;
        tp.bidg = B.a64.invdiag;
        tp.f0 = a.f;
        tp.e0 = a.phi;
        tp.bc = bc_desc(c);
        tp.nu1 = nu1;
        tp.nu2 = nu2;
        tp.nub = o.nub;
        tp.singular = c->singular ? 1 : 0;
        tp.bottom_max_iter = o.bottom_max_iter;
        tp.bottom_eps = o.bottom_eps;
        tp.iters = c->red.counters;
        tp.binv = std::is_same<T, float>::value && exact_bottom(c) ? c->bot_inv : nullptr;
        tp.omega = omega;
        launch_tail<T>(tp, c->tail_smem[tslot], c->stream);
        ++c->issued;
        return;
    }
    const OtfParams P = otf ? otf_params(c) : OtfParams{};
    Level& C = c->lev[l + 1];
    LevelArrays<T>& ac = arrays<T>(C);
    // over-relaxed finest level with the staged kernels: the last pre-smoothing colour-1
    // half-sweep writes its cells' defects, and the staged restriction forms only the colour-0
    // ones (instead of both colours cell by cell)
    float* blk = otf && !gs && nu1 > 0 && c->def_b && otf_staged(P) && C.d.split ? c->def_b
                                                                                  : nullptr;
    if (otf && C.d.split && fused_sweeps(c)) {
        // one kernel a sweep, out of place: the correction alternates between a32.phi (A) and
        // e_alt (B); the prolongation writes into whichever buffer makes the last post-smoothing
        // sweep end in A
        float* A = reinterpret_cast<float*>(a.phi);
        float* B = c->e_alt;
        const float* f = reinterpret_cast<const float*>(a.f);
        float* cur = A;
        mark(c, tm, 0);
        for (int s = 0; s < nu1; ++s) {
            float* out = cur == A ? B : A;
            launch_sweep_otf_fused(L.d, P, cur, out, f, c->stream, s == nu1 - 1 ? blk : nullptr);
            ++c->issued;
            cur = out;
        }
        mark(c, tm, 1);
        launch_resid_restrict_otf(L.d, C.d, P, cur, f, reinterpret_cast<float*>(ac.f),
                                  reinterpret_cast<float*>(ac.phi), gs && nu1 > 0, c->stream, blk);
        ++c->issued;
        mark(c, tm, 2);
        vcycle<T>(c, l + 1);
        mark(c, tm, 3);
        float* tgt = nu2 % 2 ? B : A;
        launch_prolong_add<float>(L.d, C.d, bc_desc(c), reinterpret_cast<const float*>(ac.phi),
                                  tgt, gs && nu2 > 0, c->stream, cur);
        ++c->issued;
        cur = tgt;
        mark(c, tm, 4);
        for (int s = 0; s < nu2; ++s) {
            float* out = cur == A ? B : A;
            launch_sweep_otf_fused(L.d, P, cur, out, f, c->stream);
            ++c->issued;
            cur = out;
        }
        mark(c, tm, 5);
        return;
    }
    auto sweep = [&](bool last_down) {
        for (int colour = 0; colour < 2; ++colour) {
            if (otf)
                launch_gsrb_otf(L.d, P, colour, reinterpret_cast<float*>(a.phi),
                                reinterpret_cast<const float*>(a.f), c->stream,
                                last_down && colour == 1 ? blk : nullptr);
            else
                launch_gsrb<T>(L.d, colour, a, c->stream, omega);
        }
        c->issued += 2;
    };
    mark(c, tm, 0);
    for (int s = 0; s < nu1; ++s) sweep(s == nu1 - 1);
    mark(c, tm, 1);
    if (otf)
        launch_resid_restrict_otf(L.d, C.d, P, reinterpret_cast<const float*>(a.phi),
                                  reinterpret_cast<const float*>(a.f),
                                  reinterpret_cast<float*>(ac.f), reinterpret_cast<float*>(ac.phi),
                                  gs && nu1 > 0, c->stream, blk);
    else
        launch_resid_restrict<T>(L.d, C.d, a, ac.f, ac.phi, gs && nu1 > 0, c->stream);
    ++c->issued;
    mark(c, tm, 2);   // (the restriction also zeroed the coarse correction ac.phi)
    vcycle<T>(c, l + 1);
    mark(c, tm, 3);
    // with post-smoothing, only colour-1 cells need the correction (see k_prolong_add)
    launch_prolong_add<T>(L.d, C.d, bc_desc(c), ac.phi, a.phi, gs && nu2 > 0, c->stream);
    ++c->issued;
    mark(c, tm, 4);
    for (int s = 0; s < nu2; ++s) sweep(false);
    mark(c, tm, 5);
}

// Flexible CG around the inner V-cycles: mixed precision with post-smoothing (after its last
// colour-1 half-sweep the V-cycle output satisfies L z = r on colour 1, which the Krylov kernels
// use).
bool use_krylov(const mac_ctx* c, int prec) {
    return prec == MAC_PREC_MIXED && c->o.inner_krylov && sweeps_up(c, true) > 0 &&
           c->o.inner_omega == 1.0;
}

int ensure_krylov(mac_ctx* c) {
    KrylovBufs& K = c->kry;
    if (K.p) return MAC_OK;
    const Dims& d = c->lev[0].d;
    int rc = 0;
    rc |= alloc_arr(c, &K.p, (size_t)d.ncell);
    rc |= alloc_arr(c, &K.q, (size_t)d.ncell);
    rc |= alloc_arr(c, &K.x, (size_t)d.ncell);
    rc |= alloc_arr(c, &K.w0, (size_t)d.half);
    rc |= alloc_arr(c, &K.partial, (size_t)krylov_partials(d));
    rc |= alloc_arr(c, &K.scalars, 4);
    rc |= alloc_arr(c, &K.count, 1);
    if (rc) {
        K = KrylovBufs();
        return MAC_ERR_ALLOC;
    }
    MAC_CUDA_TRY(cudaMemset(K.count, 0, sizeof(unsigned)));
    MAC_CUDA_TRY(cudaMemset(K.scalars, 0, 4 * sizeof(double)));
    return MAC_OK;
}

int inner_cycles(const mac_ctx* c, int prec) {
    return prec == MAC_PREC_FP64 ? 1 : (c->cur_inner > 1 ? c->cur_inner : 1);
}

int graph_slot(const mac_ctx* c, int prec) {
    return prec == MAC_PREC_FP64 ? 0 : inner_cycles(c, prec);
}

// One iteration of the outer loop, ending with the max-norm of the fine residual in
// red.maxbits and its copy in pinned host memory.
void issue_iteration(mac_ctx* c, int prec) {
    Level& F = c->lev[0];
    const bool tm = c->o.timing;
    cudaMemsetAsync(c->red.maxbits, 0, sizeof(unsigned long long), c->stream);
    if (prec == MAC_PREC_FP64) {
        c->vtimer = 0;
        vcycle<double>(c, 0);
        if (tm) cudaEventRecordWithFlags(c->tail[0], c->stream, cudaEventRecordExternal);
        if (tm) cudaEventRecordWithFlags(c->tail[1], c->stream, cudaEventRecordExternal);
        launch_resid_norm<double>(F.d, F.a64, c->o.nu2 > 0, c->red.maxbits, c->stream);
        ++c->issued;
    } else {
        // e (F.a32.phi) enters at zero: the residual kernel that formed this step's right-hand
        // side cleared it
        const int nv = inner_cycles(c, prec);
        if (use_krylov(c, prec)) {
            const OtfParams P = c->otf ? otf_params(c) : OtfParams{};
            for (int v = 0; v < nv; ++v) {
                c->vtimer = v;
                vcycle<float>(c, 0);
                const bool last = v + 1 == nv;
                launch_fcg_dots(F.d, c->dm, c->otf, P, F.a32, c->kry, v == 0, !last, c->stream);
                if (!last)
                    launch_fcg_update(F.d, F.a32, c->kry, v == 0, c->stream);
                else
                    launch_fcg_final(F.d, F.a64.phi, F.a32, c->kry, v == 0, c->stream);
                c->issued += 2;
                mark(c, tm, 6);
            }
            if (tm) cudaEventRecordWithFlags(c->tail[0], c->stream, cudaEventRecordExternal);
        } else {
            for (int v = 0; v < nv; ++v) {
                c->vtimer = v;
                vcycle<float>(c, 0);
            }
            if (tm) cudaEventRecordWithFlags(c->tail[0], c->stream, cudaEventRecordExternal);
            launch_accumulate(F.d, F.a64.phi, F.a32.phi, c->stream);
            ++c->issued;
        }
        if (tm) cudaEventRecordWithFlags(c->tail[1], c->stream, cudaEventRecordExternal);
        launch_resid64_to32(F.d, F.a64, F.a32.f, c->red.maxbits, c->stream, F.a32.phi);
        ++c->issued;
    }
    if (tm) cudaEventRecordWithFlags(c->tail[2], c->stream, cudaEventRecordExternal);
    cudaMemcpyAsync(c->red.h_maxbits, c->red.maxbits, sizeof(unsigned long long),
                    cudaMemcpyDeviceToHost, c->stream);
}

// Accumulate the per-class device times of the iteration that just completed.
void collect_timing(mac_ctx* c, int prec) {
    if (!c->o.timing) return;
    const int nv = inner_cycles(c, prec);
    for (int v = 0; v < nv && v < 4; ++v) {
        float t[5];
        for (int e = 0; e < 5; ++e) {
            t[e] = 0.f;
            cudaEventElapsedTime(&t[e], c->tev[v][e], c->tev[v][e + 1]);
        }
        c->ktime_ms[MAC_KT_SMOOTH] += t[0] + t[4];
        c->ktime_launches[MAC_KT_SMOOTH] +=
            (prec == MAC_PREC_MIXED && fused_sweeps(c) ? 1 : 2) *
            (sweeps_down(c, prec == MAC_PREC_MIXED) + sweeps_up(c, prec == MAC_PREC_MIXED));
        c->ktime_ms[MAC_KT_RESTRICT] += t[1];
        c->ktime_launches[MAC_KT_RESTRICT] += 1;
        c->ktime_ms[MAC_KT_COARSE] += t[2];
        c->ktime_ms[MAC_KT_PROLONG] += t[3];
        c->ktime_launches[MAC_KT_PROLONG] += 1;
        if (use_krylov(c, prec)) {
            float tk = 0.f;
            cudaEventElapsedTime(&tk, c->tev[v][5], c->tev[v][6]);
            c->ktime_ms[MAC_KT_ACCUM] += tk;
            c->ktime_launches[MAC_KT_ACCUM] += 2;
        }
    }
    float ta = 0.f, tr = 0.f;
    cudaEventElapsedTime(&ta, c->tail[0], c->tail[1]);
    cudaEventElapsedTime(&tr, c->tail[1], c->tail[2]);
    if (prec == MAC_PREC_MIXED && !use_krylov(c, prec)) {
        c->ktime_ms[MAC_KT_ACCUM] += ta;
        c->ktime_launches[MAC_KT_ACCUM] += 1;
    }
    c->ktime_ms[MAC_KT_RESID] += tr;
    c->ktime_launches[MAC_KT_RESID] += 1;
}

int get_iteration_exec(mac_ctx* c, int prec, cudaGraphExec_t* out) {
    const int slot = graph_slot(c, prec);
    if (c->vc_exec[slot]) {
        *out = c->vc_exec[slot];
        return MAC_OK;
    }
    cudaGraph_t g = nullptr;
    const long long before = c->issued;
    MAC_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    issue_iteration(c, prec);
    MAC_CUDA_TRY(cudaStreamEndCapture(c->stream, &g));
    c->graph_kernels[slot] = c->issued - before;
    c->issued = before;
    cudaGraphExec_t ex = nullptr;
    cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    MAC_CUDA_TRY(e);
    c->vc_exec[slot] = ex;
    *out = ex;
    return MAC_OK;
}

void drop_graphs(mac_ctx* c) {
    for (int s = 0; s <= kInnerGraphs; ++s)
        if (c->vc_exec[s]) {
            cudaGraphExecDestroy(c->vc_exec[s]);
            c->vc_exec[s] = nullptr;
        }
}

int run_iteration(mac_ctx* c, int prec, double* res_out) {
    if (c->o.use_graph && graph_slot(c, prec) <= kInnerGraphs) {
        cudaGraphExec_t ex;
        int rc = get_iteration_exec(c, prec, &ex);
        if (rc) return rc;
        MAC_CUDA_TRY(cudaGraphLaunch(ex, c->stream));
        c->issued += c->graph_kernels[graph_slot(c, prec)];
    } else {
        issue_iteration(c, prec);
        MAC_CUDA_TRY(cudaGetLastError());
    }
    MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    *res_out = bits_to_double(*c->red.h_maxbits);
    collect_timing(c, prec);
    return MAC_OK;
}

}  // namespace

// Inner V-cycles of the next mixed-precision refinement step: the per-V-cycle contraction seen
// in the step just run, r_new / r_old = rate^nv, taken a little pessimistically (rate^0.85),
// predicts how many V-cycles reach the target; at least 1, at most inner_max.
int next_inner(double r_old, double r_new, int nv, double target, int inner_max) {
    if (!(r_new > 0.0) || !(r_old > 0.0) || r_new >= r_old || target <= 0.0) return inner_max;
    const double log_rate = 0.85 * std::log(r_new / r_old) / nv;   // < 0
    const double need = std::log(target / r_new);                  // < 0 when not converged
    if (need >= 0.0) return 1;
    const double m = std::ceil(need / log_rate - 1e-9);
    if (!(m < inner_max)) return inner_max;
    return m < 1.0 ? 1 : (int)m;
}

// Multigrid solve on level 0 with f, coefficients and phi (level-0 layout) already in place.
// red.scalars[1] holds ||f||_inf (after mean removal).
int run_solve(mac_ctx* c, mac_stats* st) {
    const mac_opts& o = c->o;
    Level& F = c->lev[0];
    const int prec = o.precision;
    if (prec == MAC_PREC_MIXED) {
        int rc = setup_fp32_copies(c);
        if (rc) return rc;
        if (use_krylov(c, prec) && (rc = ensure_krylov(c))) return rc;
        if (c->o.inner_omega != 1.0 && c->otf && !c->def_b &&
            (rc = alloc_arr(c, &c->def_b, (size_t)F.d.half)))
            return rc;
        if (c->o.fused_sweep && c->otf && fused_plan(c) && !c->e_alt &&
            (rc = alloc_arr(c, &c->e_alt, (size_t)F.d.ncell)))
            return rc;
        if (exact_bottom(c)) {
            if (!c->inv_pending) {   // (a caller that built the levels some other way)
                int rc2 = issue_bottom_inverse(c);
                if (rc2) return rc2;
            }
            MAC_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->aux_ev[1], 0));
            c->inv_pending = false;
        }
    }
    MAC_CUDA_TRY(cudaMemcpyAsync(c->red.h_scalars, c->red.scalars, 8 * sizeof(double),
                                 cudaMemcpyDeviceToHost, c->stream));
    MAC_CUDA_TRY(cudaMemcpyAsync(c->red.h_counters, c->red.counters, 4 * sizeof(int),
                                 cudaMemcpyDeviceToHost, c->stream));
    MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (c->red.h_counters[1]) return MAC_ERR_BAD_DENSITY;
    const double fnorm = c->red.h_scalars[1];
    st->fnorm = fnorm;
    if (!std::isfinite(fnorm)) return MAC_ERR_NONFINITE;
    MAC_CUDA_TRY(cudaMemsetAsync(c->red.counters, 0, sizeof(int), c->stream));
    const bool mean_pending = c->mean_pending;
    c->mean_pending = false;
    if (fnorm == 0.0) {
        MAC_CUDA_TRY(cudaMemsetAsync(F.a64.phi, 0, sizeof(double) * F.d.ncell, c->stream));
        st->rel_resid = 0.0;
        return MAC_OK;
    }
    auto converged = [&](double r) {
        return r <= o.rel_eps * fnorm || (o.abs_eps > 0.0 && r <= o.abs_eps);
    };
    // initial residual of the caller's guess (both colours); f loses its mean (singular problem)
    // on the way.  A guess that is +0 everywhere (the usual zero start) leaves r = f - mean, whose
    // max-norm fnorm already is.
    unsigned long long guess_bits;
    std::memcpy(&guess_bits, &c->red.h_scalars[5], sizeof(guess_bits));
    const bool zero_guess = guess_bits == 0ull;
    double res;
    MAC_CUDA_TRY(cudaMemsetAsync(c->red.maxbits, 0, sizeof(unsigned long long), c->stream));
    if (prec == MAC_PREC_MIXED && zero_guess) {
        launch_first_resid_zero(F.d, F.a64.f, mean_pending ? c->red.scalars : nullptr, F.a32.f,
                                F.a32.phi, c->red.maxbits, c->stream);
        ++c->issued;
    } else {
        if (mean_pending) {
            launch_sub_mean(c);
            ++c->issued;
        }
        if (prec == MAC_PREC_FP64) {
            if (!zero_guess) {
                launch_resid_norm<double>(F.d, F.a64, false, c->red.maxbits, c->stream);
                ++c->issued;
            }
        } else {
            launch_resid64_to32(F.d, F.a64, F.a32.f, c->red.maxbits, c->stream, F.a32.phi);
            ++c->issued;
        }
    }
    MAC_CUDA_TRY(cudaGetLastError());
    if (prec == MAC_PREC_FP64 && zero_guess) {
        res = fnorm;   // max |f - mean| (rounding is monotone: equal to the cell-wise maximum)
    } else {
        MAC_CUDA_TRY(cudaMemcpyAsync(c->red.h_maxbits, c->red.maxbits, sizeof(unsigned long long),
                                     cudaMemcpyDeviceToHost, c->stream));
        MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
        res = bits_to_double(*c->red.h_maxbits);
    }
    st->resid0 = res;
    if (!std::isfinite(res)) return MAC_ERR_NONFINITE;
    int it = 0, nv_total = 0;
    const int inner_max = o.inner_vcycles > 1 ? o.inner_vcycles : 1;
    const double target = std::max(o.rel_eps * fnorm, o.abs_eps > 0.0 ? o.abs_eps : 0.0);
    c->cur_inner = inner_max;
    while (!converged(res) && it < o.max_vcycles) {
        const double res_prev = res;
        const int nv = inner_cycles(c, prec);
        int rc = run_iteration(c, prec, &res);
        if (rc) return rc;
        ++it;
        nv_total += nv;
        if (st->nhist < 64) st->hist[st->nhist++] = res / fnorm;
        if (!std::isfinite(res)) {
            st->vcycles = nv_total;
            st->rel_resid = res / fnorm;
            // a staged kernel that gave up a wait left its part of the sweep undone: report that
            MAC_CUDA_TRY(cudaMemcpyAsync(c->red.h_counters, c->red.counters, 3 * sizeof(int),
                                         cudaMemcpyDeviceToHost, c->stream));
            MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
            return c->red.h_counters[2] ? MAC_ERR_DEVICE_TIMEOUT : MAC_ERR_NONFINITE;
        }
        if (prec == MAC_PREC_MIXED && o.adaptive_inner)
            c->cur_inner = next_inner(res_prev, res, nv, target, inner_max);
    }
    st->vcycles = nv_total;
    st->refine_iters = prec == MAC_PREC_MIXED ? it : 0;
    st->rel_resid = res / fnorm;
    MAC_CUDA_TRY(cudaMemcpyAsync(c->red.h_counters, c->red.counters, 3 * sizeof(int),
                                 cudaMemcpyDeviceToHost, c->stream));
    MAC_CUDA_TRY(cudaStreamSynchronize(c->stream));
    st->bottom_iters = c->red.h_counters[0];
    if (c->red.h_counters[2]) return MAC_ERR_DEVICE_TIMEOUT;
    return converged(res) ? MAC_OK : MAC_ERR_NOT_CONVERGED;
}

}  // namespace mac

using namespace mac;

namespace {

int nlevels_for(const mac_ctx* c) {
    // FBoxLib rule: coarsen every box by 2 while all of its extents stay even and >= 2 after
    // halving (Docs/mg/mg.tex:227-236).
    int cmin = 1 << 30;
    for (int b = 0; b < c->g.nboxes; ++b)
        for (int d = 0; d < c->dm; ++d) {
            int e = c->box_hi[3 * b + d] - c->box_lo[3 * b + d] + 1;
            int k = 0;
            while (e % 2 == 0 && e / 2 >= 2) {
                e /= 2;
                ++k;
            }
            cmin = std::min(cmin, k);
        }
    int nl = 1 + (cmin == (1 << 30) ? 0 : cmin);
    if (c->o.max_levels > 0) nl = std::min(nl, c->o.max_levels);
    return std::min(nl, kMaxLevels);
}

int validate_geom(const mac_geom* g) {
    if (!g || (g->dm != 2 && g->dm != 3) || g->nboxes <= 0 || !g->box_lo || !g->box_hi)
        return MAC_ERR_INVALID;
    for (int d = 0; d < g->dm; ++d) {
        if (g->domain_hi[d] < g->domain_lo[d] || !(g->dx[d] > 0.0)) return MAC_ERR_INVALID;
        const int bl = g->bc_lo[d], bh = g->bc_hi[d];
        if (bl != MAC_BC_PER && bl != MAC_BC_DIR && bl != MAC_BC_NEU) return MAC_ERR_INVALID;
        if (bh != MAC_BC_PER && bh != MAC_BC_DIR && bh != MAC_BC_NEU) return MAC_ERR_INVALID;
        if ((bl == MAC_BC_PER) != (bh == MAC_BC_PER)) return MAC_ERR_INVALID;
    }
    // boxes inside the domain and tiling it exactly (cell counts add up, no overlap by volume)
    long long vol = 0, dom = 1;
    for (int d = 0; d < g->dm; ++d) dom *= (long long)(g->domain_hi[d] - g->domain_lo[d] + 1);
    for (int b = 0; b < g->nboxes; ++b) {
        long long v = 1;
        for (int d = 0; d < g->dm; ++d) {
            const int lo = g->box_lo[3 * b + d], hi = g->box_hi[3 * b + d];
            if (hi < lo || lo < g->domain_lo[d] || hi > g->domain_hi[d]) return MAC_ERR_INVALID;
            v *= (long long)(hi - lo + 1);
        }
        vol += v;
    }
    if (vol != dom) return MAC_ERR_INVALID;
    if (dom >= (1ll << 31) - 1) return MAC_ERR_UNSUPPORTED;
    return MAC_OK;
}

int check_opts(const mac_opts* o) {
    if (!o) return MAC_ERR_INVALID;
    if (o->precision != MAC_PREC_FP64 && o->precision != MAC_PREC_MIXED) return MAC_ERR_INVALID;
    if (o->nu1 < 0 || o->nu2 < 0 || o->nub < 0 || o->max_vcycles < 0 || o->bottom_max_iter < 0)
        return MAC_ERR_INVALID;
    if (o->inner_nu1 < -1 || o->inner_nu2 < -1) return MAC_ERR_INVALID;
    if (!(o->inner_omega > 0.0 && o->inner_omega < 2.0)) return MAC_ERR_INVALID;
    if (!(o->rel_eps >= 0.0)) return MAC_ERR_INVALID;
    if (!(o->wait_limit_s > 0.0 && o->wait_limit_s <= 10.0)) return MAC_ERR_INVALID;
    if (o->inject_wait_expiry != 0 && o->inject_wait_expiry != 1) return MAC_ERR_INVALID;
    if (o->fused_sweep != 0 && o->fused_sweep != 1) return MAC_ERR_INVALID;
    return MAC_OK;
}

int ctx_alloc(mac_ctx* c) {
    int rc = 0;
    const size_t N = (size_t)c->n[0] * c->n[1] * c->n[2];
    c->lev.assign(c->nlevels, Level());
    int n[3] = {c->n[0], c->n[1], c->n[2]};
    double h[3] = {c->dx[0], c->dx[1], c->dx[2]};
    for (int l = 0; l < c->nlevels; ++l) {
        Level& L = c->lev[l];
        L.d.n0 = n[0];
        L.d.n1 = n[1];
        L.d.n2 = n[2];
        L.d.ncell = n[0] * n[1] * n[2];
        L.d.split = (l < c->nlevels - 1) ? 1 : 0;
        L.d.hn0 = n[0] / 2;
        L.d.half = L.d.ncell / 2;
        L.d.rz = c->dm == 3 ? 2 : 1;
        for (int d = 0; d < 3; ++d) L.h[d] = h[d];
        if (L.d.split && (n[0] % 2 || n[1] % 2 || (c->dm == 3 && n[2] % 2))) return MAC_ERR_UNSUPPORTED;
        const size_t nc = L.d.ncell;
        rc |= alloc_arr(c, &L.a64.phi, nc);
        rc |= alloc_arr(c, &L.a64.f, nc);
        rc |= alloc_arr(c, &L.a64.bx, nc);
        rc |= alloc_arr(c, &L.a64.by, nc);
        rc |= alloc_arr(c, &L.a64.bz, nc);
        rc |= alloc_arr(c, &L.a64.diag, nc);
        rc |= alloc_arr(c, &L.a64.invdiag, nc);
        for (int d = 0; d < c->dm; ++d)
            for (int s = 0; s < 2; ++s) {
                const int bc = s ? c->bc_hi[d] : c->bc_lo[d];
                if (bc != MAC_BC_DIR) continue;
                const int p0 = d == 0 ? 1 : 0, p1 = d == 2 ? 1 : 2;
                rc |= alloc_arr(c, &L.wall[d][s], (size_t)n[p0] * n[p1]);
            }
        if (rc) return MAC_ERR_ALLOC;
        if (l + 1 < c->nlevels) {
            n[0] /= 2;
            n[1] /= 2;
            if (c->dm == 3) n[2] /= 2;
            h[0] *= 2;
            h[1] *= 2;
            if (c->dm == 3) h[2] *= 2;
        }
    }
    // FP32 copies for the mixed-precision inner cycle (precision can change per call)
    for (auto& L : c->lev) {
        rc = alloc_level_fp32(c, L);
        if (rc) return rc;
    }
    // z coefficients of a 2-D problem stay zero
    if (c->dm == 2)
        for (auto& L : c->lev) {
            MAC_CUDA_TRY(cudaMemset(L.a64.bz, 0, sizeof(double) * L.d.ncell));
            MAC_CUDA_TRY(cudaMemset(L.a32.bz, 0, sizeof(float) * L.d.ncell));
        }
    const Level& B = c->lev[c->nlevels - 1];
    if (B.d.ncell > kBottomMaxCells) return MAC_ERR_UNSUPPORTED;
    // single-CTA tail plans: from the first level >= 1 that is small enough (FP32 <= 4096 cells,
    // FP64 <= 512: one SM's FP64 rate) and whose tail fits in shared memory
    for (int slot = 0; slot < 2; ++slot) {
        const int limit = slot ? 4096 : 512;
        c->tail_start[slot] = -1;
        if (B.d.ncell > 4096) continue;
        for (int l = 1; l < c->nlevels - 1; ++l) {
            if (c->lev[l].d.ncell > limit || c->nlevels - 1 - l > kTailMaxLevels) continue;
            Dims ds[kTailMaxLevels];
            for (int q = 0; q < c->nlevels - 1 - l; ++q) ds[q] = c->lev[l + q].d;
            const size_t bytes = slot ? tail_smem_bytes<float>(ds, c->nlevels - 1 - l, B.d)
                                      : tail_smem_bytes<double>(ds, c->nlevels - 1 - l, B.d);
            if (bytes > (size_t)kTailSmemMax) continue;
            c->tail_start[slot] = l;
            c->tail_smem[slot] = bytes;
            break;
        }
    }
    rc |= alloc_arr(c, &c->bottom_scratch, (size_t)(2 + kBotScrPerCell) * B.d.ncell);
    if (c->tail_start[1] >= 0 && B.d.ncell <= kDenseBottomMax)
        rc |= alloc_arr(c, &c->bot_inv, (size_t)B.d.ncell * B.d.ncell);
    for (int d = 0; d < c->dm; ++d) {
        const size_t nf = (size_t)(c->n[0] + (d == 0)) * (c->n[1] + (d == 1)) * (c->n[2] + (d == 2));
        rc |= alloc_arr(c, &c->u[d], nf);
    }
    rc |= alloc_arr(c, &c->rho, N);
    rc |= alloc_arr(c, &c->rhs, N);
    rc |= alloc_arr(c, &c->phin, N);
    rc |= alloc_arr(c, &c->scratch, N);
    rc |= alloc_arr(c, &c->base1d, (size_t)4 * (c->n[c->va] + 1));
    const int nr = c->n[c->va];
    rc |= alloc_arr(c, &c->beta0, (size_t)nr);
    rc |= alloc_arr(c, &c->beta0e, (size_t)nr + 1);
    rc |= alloc_arr(c, &c->b0tab, (size_t)kTabCount * (nr + 1));
    rc |= alloc_arr(c, &c->fac32, (size_t)kOtfTables * (nr + 1));
    rc |= alloc_arr(c, &c->rho32, N);
    const Grid3 rg = rhs_grid(c->n);
    const int nbp = (int)(rg.grid.x * rg.grid.y * rg.grid.z);
    c->red.nblocks_partial = nbp;
    rc |= alloc_arr(c, &c->red.partial, (size_t)kRhsPartials * nbp);
    rc |= alloc_arr(c, &c->red.scalars, 8);
    rc |= alloc_arr(c, &c->red.counters, 4);
    rc |= alloc_arr(c, &c->red.maxbits, 1);
    if (rc) return MAC_ERR_ALLOC;
    {
        int dev = 0;
        MAC_CUDA_TRY(cudaGetDevice(&dev));
        MAC_CUDA_TRY(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev));
        plan_otf_tile(c->lev[0].d, c->dm, c->sms, c->otf_tile);
    }
    MAC_CUDA_TRY(cudaMallocHost(&c->red.h_maxbits, sizeof(unsigned long long)));
    MAC_CUDA_TRY(cudaMallocHost(&c->red.h_scalars, 8 * sizeof(double)));
    MAC_CUDA_TRY(cudaMallocHost(&c->red.h_counters, 4 * sizeof(int)));
    c->box_table_cap = 16 * c->g.nboxes;
    MAC_CUDA_TRY(cudaMallocHost(&c->h_boxes, sizeof(BoxDesc) * c->box_table_cap));
    rc |= alloc_arr(c, &c->d_boxes, (size_t)c->box_table_cap);
    if (rc) return MAC_ERR_ALLOC;
    for (int e = 0; e < 4; ++e) MAC_CUDA_TRY(cudaEventCreate(&c->ev[e]));
    for (int v = 0; v < 4; ++v)
        for (int e = 0; e < 8; ++e) MAC_CUDA_TRY(cudaEventCreate(&c->tev[v][e]));
    for (int e = 0; e < 3; ++e) MAC_CUDA_TRY(cudaEventCreate(&c->tail[e]));
    MAC_CUDA_TRY(cudaMemset(c->red.counters, 0, 4 * sizeof(int)));
    // copy-engine stream of host-pointer calls (independent of the legacy stream) and its events
    MAC_CUDA_TRY(cudaStreamCreateWithFlags(&c->xfer, cudaStreamNonBlocking));
    MAC_CUDA_TRY(cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking));
    for (cudaEvent_t& e : c->aux_ev) MAC_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (cudaEvent_t& e : c->xev) MAC_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return MAC_OK;
}

void ctx_free(mac_ctx* c) {
    amr_release(c);
    hg_release(c);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->xfer) cudaStreamSynchronize(c->xfer);
    if (c->aux) cudaStreamSynchronize(c->aux);
    drop_graphs(c);
    for (void* p : c->allocations) cudaFree(p);
    c->allocations.clear();
    if (c->staging) cudaFree(c->staging);
    if (c->red.h_maxbits) cudaFreeHost(c->red.h_maxbits);
    if (c->red.h_scalars) cudaFreeHost(c->red.h_scalars);
    if (c->red.h_counters) cudaFreeHost(c->red.h_counters);
    if (c->h_boxes) cudaFreeHost(c->h_boxes);
    for (int e = 0; e < 4; ++e)
        if (c->ev[e]) cudaEventDestroy(c->ev[e]);
    for (int v = 0; v < 4; ++v)
        for (int e = 0; e < 8; ++e)
            if (c->tev[v][e]) cudaEventDestroy(c->tev[v][e]);
    for (int e = 0; e < 3; ++e)
        if (c->tail[e]) cudaEventDestroy(c->tail[e]);
    for (cudaEvent_t& e : c->xev)
        if (e) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    if (c->xfer) cudaStreamDestroy(c->xfer);
    c->xfer = nullptr;
    for (cudaEvent_t& e : c->aux_ev)
        if (e) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    if (c->aux) cudaStreamDestroy(c->aux);
    c->aux = nullptr;
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    c->stream = nullptr;
}

// Copy a 1-D beta0 array (host or device) into the context.
int load_beta0_impl(mac_ctx* c, int ptr_kind, const double* b0, const double* b0e) {
    const int nr = c->n[c->va];
    const cudaMemcpyKind k = ptr_kind == MAC_PTR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    MAC_CUDA_TRY(cudaMemcpyAsync(c->beta0, b0, sizeof(double) * nr, k, c->stream));
    MAC_CUDA_TRY(cudaMemcpyAsync(c->beta0e, b0e, sizeof(double) * (nr + 1), k, c->stream));
    return MAC_OK;
}

// Per-call operator state: alpha on/off (Helmholtz) and whether the problem is singular.
// CUDA graphs bake the singular flag into the bottom solve, so they are dropped on a change.
int set_otf(mac_ctx* c, bool on) {
    if (on != c->otf) drop_graphs(c);
    c->otf = on;
    return MAC_OK;
}

int set_call_state_impl(mac_ctx* c, bool with_alpha) {
    for (auto& L : c->lev) {
        if (with_alpha && !L.alpha_store) {
            int rc = alloc_arr(c, &L.alpha_store, (size_t)L.d.ncell);
            if (rc) return rc;
        }
        L.alpha = with_alpha ? L.alpha_store : nullptr;
    }
    const bool sing = c->geom_singular && !with_alpha;
    if (sing != c->singular) drop_graphs(c);
    c->singular = sing;
    return MAC_OK;
}

// The projection on whole-domain device arrays already in c->u / c->rho / rhs / phin.
int core_macproject(mac_ctx* c, const double* macrhs, bool have_beta0, mac_stats* st,
                    const std::function<int()>* before_rhs = nullptr,
                    const std::function<int()>* before_phi = nullptr,
                    const std::function<int()>* after_phi = nullptr,
                    const std::function<int(int)>* after_dir = nullptr) {
    Level& F = c->lev[0];
    cudaEventRecord(c->ev[0], c->stream);
    int rc = set_call_state_impl(c, false);
    if (rc) return rc;
    set_otf(c, c->o.precision == MAC_PREC_MIXED);
    rc = setup_fine_coefficients(c, have_beta0 ? c->beta0 : nullptr, have_beta0 ? c->beta0e : nullptr);
    if (rc) return rc;
    rc = setup_coarse_levels(c);
    if (rc) return rc;
    if (before_rhs && (rc = (*before_rhs)())) return rc;
    if (before_phi && (rc = (*before_phi)())) return rc;
    rc = setup_rhs(c, macrhs, have_beta0, c->phin);   // also moves phi into the level-0 layout
    if (rc) return rc;
    cudaEventRecord(c->ev[1], c->stream);
    const long long setup_kernels = c->issued;
    const int solve_rc = run_solve(c, st);
    if (solve_rc != MAC_OK && solve_rc != MAC_ERR_NOT_CONVERGED) return solve_rc;
    cudaEventRecord(c->ev[2], c->stream);
    const long long before_corr = c->issued;
    // the x-direction correction also returns phi to the natural layout; phi's copy-back (host
    // pointers) starts right after it
    const std::function<int(int)> dir_hook = [&](int d) {
        int r = MAC_OK;
        if (d == 0 && after_phi) r = (*after_phi)();
        if (!r && after_dir) r = (*after_dir)(d);
        return r;
    };
    rc = correct_velocity(c, have_beta0, &dir_hook, c->phin);
    if (rc) return rc;
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

void fill_common_stats(mac_ctx* c, mac_stats* st) {
    st->nlevels = c->nlevels;
    c->issued = 0;
    for (int k = 0; k < MAC_KT_NCLASS; ++k) {
        c->ktime_ms[k] = 0.0;
        c->ktime_launches[k] = 0;
    }
}

void finish_stats(mac_ctx* c, mac_stats* st) {
    st->launches = c->issued;
    for (int k = 0; k < MAC_KT_NCLASS; ++k) {
        st->ktime_ms[k] = c->ktime_ms[k];
        st->ktime_launches[k] = c->ktime_launches[k];
    }
}

void report(const mac_ctx* c, const char* what, const mac_stats* st) {
    if (c->o.verbose <= 0) return;
    std::fprintf(stderr,
                 "[maestro_mac] %s: status %d (%s) prec=%s levels=%d vcycles=%d rel_resid=%.3e "
                 "setup=%.3f ms solve=%.3f ms total=%.3f ms\n",
                 what, st->status, mac_strerror(st->status),
                 c->o.precision == MAC_PREC_MIXED ? "mixed" : "fp64", st->nlevels, st->vcycles,
                 st->rel_resid, st->setup_ms, st->solve_ms, st->total_ms);
}

}  // namespace

namespace mac {
// (launched outside a stream capture: the V-cycle's own class-timing events, which are
// recorded as nodes of its captured graph, stay off)
int level0_fp64_vcycle(mac_ctx* c) {
    const int tm = c->o.timing;
    c->o.timing = 0;
    vcycle<double>(c, 0);
    c->o.timing = tm;
    MAC_CUDA_TRY(cudaGetLastError());
    return MAC_OK;
}
int level0_fp32_vcycle(mac_ctx* c) {
    const int tm = c->o.timing;
    c->o.timing = 0;
    vcycle<float>(c, 0);
    c->o.timing = tm;
    MAC_CUDA_TRY(cudaGetLastError());
    return MAC_OK;
}
int forward_projection(mac_ctx* c, const double* macrhs, bool have_beta0, mac_stats* st) {
    return core_macproject(c, macrhs, have_beta0, st);
}
int set_call_state(mac_ctx* c, bool with_alpha) { return set_call_state_impl(c, with_alpha); }
int set_otf_mode(mac_ctx* c, bool on) { return set_otf(c, on); }
void report_call(const mac_ctx* c, const char* what, const mac_stats* st) { report(c, what, st); }

int issue_bottom_inverse(mac_ctx* c) {
    // an inverse issued by a call that stopped before its solve may still read the operator the
    // main stream is about to rebuild
    if (c->inv_pending) MAC_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->aux_ev[1], 0));
    c->inv_pending = false;
    if (c->o.precision != MAC_PREC_MIXED || !exact_bottom(c)) return MAC_OK;
    const Level& B = c->lev[c->nlevels - 1];
    MAC_CUDA_TRY(cudaEventRecord(c->aux_ev[0], c->stream));
    MAC_CUDA_TRY(cudaStreamWaitEvent(c->aux, c->aux_ev[0], 0));
    launch_bottom_inverse(B.d, B.a64.bx, B.a64.by, B.a64.bz, B.a64.diag, c->singular, c->bot_inv,
                          c->aux);
    MAC_CUDA_TRY(cudaGetLastError());
    ++c->issued;
    MAC_CUDA_TRY(cudaEventRecord(c->aux_ev[1], c->aux));
    c->inv_pending = true;
    return MAC_OK;
}
int load_beta0(mac_ctx* c, int ptr_kind, const double* b0, const double* b0e) {
    return load_beta0_impl(c, ptr_kind, b0, b0e);
}
void begin_call_stats(mac_ctx* c, mac_stats* st) { fill_common_stats(c, st); }
void end_call_stats(mac_ctx* c, mac_stats* st) { finish_stats(c, st); }
}  // namespace mac

extern "C" {

void mac_default_opts(mac_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->precision = MAC_PREC_FP64;
    o->use_alt_energy_fix = 0;
    o->rel_eps = 1e-10;   // min(eps_mac * 10^(nlevs-1), eps_mac_max), one AMR level
    o->abs_eps = -1.0;
    o->max_vcycles = 100;
    o->nu1 = 2;
    o->nu2 = 2;
    o->nub = 10;
    o->bottom_eps = 1e-3;
    o->bottom_max_iter = 200;
    o->max_levels = 0;
    o->use_graph = 1;
    o->verbose = 0;
    o->timing = 0;
    o->inner_vcycles = 3;
    o->coarse_tail = 1;
    o->adaptive_inner = 1;
    o->inner_krylov = 0;
    o->inner_nu1 = 2;
    o->inner_nu2 = 1;
    o->inner_exact_bottom = 1;
    o->inner_omega = 1.25;
    o->wait_limit_s = 1.0;
    o->inject_wait_expiry = 0;
    o->fused_sweep = 0;
}

const char* mac_strerror(int code) {
    switch (code) {
        case MAC_OK: return "ok";
        case MAC_ERR_INVALID: return "invalid argument";
        case MAC_ERR_CUDA: return g_last_cuda.empty() ? "CUDA error" : g_last_cuda.c_str();
        case MAC_ERR_NOT_CONVERGED: return "multigrid did not reach the tolerance within max_vcycles";
        case MAC_ERR_NONFINITE: return "non-finite value in the right-hand side or residual";
        case MAC_ERR_ALLOC: return "device allocation failed";
        case MAC_ERR_UNSUPPORTED:
            return "unsupported geometry (every level but the coarsest needs even extents; the "
                   "coarsest level must hold at most 65536 cells; at least two MG levels)";
        case MAC_ERR_BAD_DENSITY: return "density <= 0 or non-finite";
        case MAC_ERR_TOO_LARGE: return "size above the fixed limit of this entry point";
        case MAC_ERR_DEVICE_TIMEOUT:
            return "a kernel gave up waiting (about 1 s) for its own asynchronous copies";
        default: return "unknown status";
    }
}

const char* mac_version(void) { return "maestro_gb300 mac 0.1 (sm_103a)"; }

int mac_ctx_create(mac_ctx** out, const mac_geom* g, const mac_opts* o, void* cuda_stream) {
    if (!out) return MAC_ERR_INVALID;
    *out = nullptr;
    int rc = validate_geom(g);
    if (rc) return rc;
    mac_opts oo;
    if (o) {
        oo = *o;
    } else {
        mac_default_opts(&oo);
    }
    rc = check_opts(&oo);
    if (rc) return rc;
    mac_ctx* c = new mac_ctx();
    c->g = *g;
    c->o = oo;
    c->box_lo.assign(g->box_lo, g->box_lo + 3 * g->nboxes);
    c->box_hi.assign(g->box_hi, g->box_hi + 3 * g->nboxes);
    c->g.box_lo = c->box_lo.data();
    c->g.box_hi = c->box_hi.data();
    c->dm = g->dm;
    for (int d = 0; d < 3; ++d) {
        c->n[d] = d < g->dm ? g->domain_hi[d] - g->domain_lo[d] + 1 : 1;
        c->bc_lo[d] = d < g->dm ? g->bc_lo[d] : MAC_BC_NEU;
        c->bc_hi[d] = d < g->dm ? g->bc_hi[d] : MAC_BC_NEU;
        c->dx[d] = d < g->dm ? g->dx[d] : 1.0;
    }
    c->va = g->dm - 1;
    bool has_dir = false;
    for (int d = 0; d < g->dm; ++d) has_dir = has_dir || c->bc_lo[d] == MAC_BC_DIR || c->bc_hi[d] == MAC_BC_DIR;
    c->singular = !has_dir;
    c->geom_singular = !has_dir;
    c->stream = (cudaStream_t)cuda_stream;
    if (!c->stream) {
        // graph capture is not possible on the legacy NULL stream; a blocking stream keeps the
        // legacy-stream ordering of the caller's work
        if (cudaStreamCreate(&c->stream) != cudaSuccess) {
            cudaGetLastError();
            delete c;
            return MAC_ERR_CUDA;
        }
        c->own_stream = true;
    }
    c->nlevels = nlevels_for(c);
    if (c->nlevels < 2) {
        if (c->own_stream) cudaStreamDestroy(c->stream);
        delete c;
        return MAC_ERR_UNSUPPORTED;
    }
    rc = prepare_kernels();
    if (!rc) rc = prepare_tail_kernels();
    if (!rc) rc = ctx_alloc(c);
    if (rc) {
        ctx_free(c);
        delete c;
        return rc;
    }
    *out = c;
    return MAC_OK;
}

int mac_ctx_destroy(mac_ctx* c) {
    if (!c) return MAC_ERR_INVALID;
    ctx_free(c);
    delete c;
    return MAC_OK;
}

int mac_ctx_set_opts(mac_ctx* c, const mac_opts* o) {
    if (!c) return MAC_ERR_INVALID;
    int rc = check_opts(o);
    if (rc) return rc;
    if (o->max_levels != c->o.max_levels) return MAC_ERR_INVALID;   // hierarchy is fixed
    drop_graphs(c);
    c->o = *o;
    return MAC_OK;
}

int mac_ctx_levels(const mac_ctx* c, int* n_out) {
    if (!c) return MAC_ERR_INVALID;
    if (n_out)
        for (int l = 0; l < c->nlevels; ++l) {
            n_out[3 * l + 0] = c->lev[l].d.n0;
            n_out[3 * l + 1] = c->lev[l].d.n1;
            n_out[3 * l + 2] = c->lev[l].d.n2;
        }
    return c->nlevels;
}

int mac_macproject_dense(mac_ctx* c, double* ux, double* uy, double* uz, double* phi,
                         const double* rho, const double* macrhs, const double* beta0,
                         const double* beta0_edge, mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if (!c || !ux || !uy || (c->dm == 3 && !uz) || !phi || !rho) return st->status = MAC_ERR_INVALID;
    if ((beta0 == nullptr) != (beta0_edge == nullptr)) return st->status = MAC_ERR_INVALID;
    const auto t0 = std::chrono::steady_clock::now();
    fill_common_stats(c, st);
    double* saved_u[3] = {c->u[0], c->u[1], c->u[2]};
    double* saved_rho = c->rho;
    double* saved_phin = c->phin;
    c->u[0] = ux;
    c->u[1] = uy;
    c->u[2] = c->dm == 3 ? uz : nullptr;
    c->rho = const_cast<double*>(rho);
    c->phin = phi;
    int rc = MAC_OK;
    if (beta0) rc = load_beta0_impl(c, MAC_PTR_DEVICE, beta0, beta0_edge);
    if (!rc) rc = core_macproject(c, macrhs, beta0 != nullptr, st);
    c->u[0] = saved_u[0];
    c->u[1] = saved_u[1];
    c->u[2] = saved_u[2];
    c->rho = saved_rho;
    c->phin = saved_phin;
    st->status = rc;
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    finish_stats(c, st);
    report(c, "macproject_dense", st);
    return rc;
}

int mac_macproject(mac_ctx* c, int ptr_kind, double* const* umac, int ng_u, double* const* phi,
                   int ng_phi, const double* const* rho, int ng_rho, int rho_ncomp, int rho_comp,
                   const double* const* macrhs, int ng_rhs, const double* beta0_1d,
                   const double* beta0_1d_edge, mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if (!c || !umac || !phi || !rho) return st->status = MAC_ERR_INVALID;
    if (ptr_kind != MAC_PTR_HOST && ptr_kind != MAC_PTR_DEVICE) return st->status = MAC_ERR_INVALID;
    if (ng_u < 0 || ng_phi < 0 || ng_rho < 0 || ng_rhs < 0 || rho_ncomp < 1 || rho_comp < 0 ||
        rho_comp >= rho_ncomp)
        return st->status = MAC_ERR_INVALID;
    if ((beta0_1d == nullptr) != (beta0_1d_edge == nullptr)) return st->status = MAC_ERR_INVALID;
    const int nb = c->g.nboxes;
    for (int b = 0; b < nb; ++b) {
        if (!phi[b] || !rho[b] || (macrhs && !macrhs[b])) return st->status = MAC_ERR_INVALID;
        for (int d = 0; d < c->dm; ++d)
            if (!umac[d * nb + b]) return st->status = MAC_ERR_INVALID;
    }
    const auto t0 = std::chrono::steady_clock::now();
    fill_common_stats(c, st);
    int rc = MAC_OK;
    if (ptr_kind == MAC_PTR_HOST) {
        size_t need = host_fab_elems(c, -1, ng_rho) + host_fab_elems(c, -1, ng_phi);
        for (int d = 0; d < c->dm; ++d) need += host_fab_elems(c, d, ng_u);
        if (macrhs) need += host_fab_elems(c, -1, ng_rhs);
        rc = staging_reserve(c, need);
    }
    // Host pointers: every input's copy is queued on the copy engines at once, in the order the
    // setup consumes them (rho, velocities, rhs, phi); each gather kernel waits only for its own
    // array, so the coefficient setup runs while the later arrays are still in flight.
    PendingGather g_rho, g_u[3], g_rhs, g_phi;
    // beta0 first: its small copy must not queue behind the bulk inputs on the copy engine
    if (!rc && beta0_1d) rc = load_beta0_impl(c, ptr_kind, beta0_1d, beta0_1d_edge);
    if (!rc) rc = gather_begin(c, ptr_kind, rho, ng_rho, rho_ncomp, rho_comp, -1, c->rho, &g_rho);
    for (int d = 0; d < c->dm && !rc; ++d)
        rc = gather_begin(c, ptr_kind, (const double* const*)(umac + d * nb), ng_u, 1, 0, d, c->u[d],
                          &g_u[d]);
    if (!rc && macrhs) rc = gather_begin(c, ptr_kind, macrhs, ng_rhs, 1, 0, -1, c->rhs, &g_rhs);
    if (!rc) rc = gather_begin(c, ptr_kind, (const double* const*)phi, ng_phi, 1, 0, -1, c->phin,
                               &g_phi);
    if (!rc) rc = gather_end(c, g_rho);
    const std::function<int()> before_rhs = [&]() {
        for (int d = 0; d < c->dm; ++d) {
            int r = gather_end(c, g_u[d]);
            if (r) return r;
        }
        return macrhs ? gather_end(c, g_rhs) : MAC_OK;
    };
    const std::function<int()> before_phi = [&]() { return gather_end(c, g_phi); };
    // outputs go back as soon as each is final: phi before the velocity correction, each
    // velocity component right after its correction kernel
    const std::function<int()> after_phi = [&]() {
        return scatter_cells(c, ptr_kind, phi, ng_phi, c->phin);
    };
    const std::function<int(int)> after_dir = [&](int d) {
        return scatter_faces(c, ptr_kind, umac + d * nb, ng_u, d, c->u[d]);
    };
    int solve_rc = MAC_OK;
    if (!rc) {
        solve_rc = core_macproject(c, macrhs ? c->rhs : nullptr, beta0_1d != nullptr, st,
                                   &before_rhs, &before_phi, &after_phi, &after_dir);
        if (solve_rc != MAC_OK && solve_rc != MAC_ERR_NOT_CONVERGED) rc = solve_rc;
    }
    {
        cudaError_t e = cudaStreamSynchronize(c->xfer);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess && !rc) {
            set_last_cuda_error(e, "cudaStreamSynchronize", __FILE__, __LINE__);
            rc = MAC_ERR_CUDA;
        }
    }
    if (!rc) rc = solve_rc;
    st->status = rc;
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    finish_stats(c, st);
    report(c, "macproject", st);
    return rc;
}

int mac_multigrid(mac_ctx* c, int ptr_kind, const double* const* rh, int ng_rh,
                  double* const* phi, int ng_phi, const double* const* alpha, int ng_alpha,
                  const double* const* beta, int ng_beta, mac_stats* stats) {
    mac_stats local;
    mac_stats* st = stats ? stats : &local;
    std::memset(st, 0, sizeof(*st));
    if (!c || !rh || !phi || !beta) return st->status = MAC_ERR_INVALID;
    if (ptr_kind != MAC_PTR_HOST && ptr_kind != MAC_PTR_DEVICE) return st->status = MAC_ERR_INVALID;
    if (ng_rh < 0 || ng_phi < 0 || ng_alpha < 0 || ng_beta < 0) return st->status = MAC_ERR_INVALID;
    const int nb = c->g.nboxes;
    for (int b = 0; b < nb; ++b) {
        if (!rh[b] || !phi[b] || (alpha && !alpha[b])) return st->status = MAC_ERR_INVALID;
        for (int d = 0; d < c->dm; ++d)
            if (!beta[d * nb + b]) return st->status = MAC_ERR_INVALID;
    }
    const auto t0 = std::chrono::steady_clock::now();
    fill_common_stats(c, st);
    Level& F = c->lev[0];
    int rc = set_call_state_impl(c, alpha != nullptr);
    set_otf(c, false);
    if (!rc && ptr_kind == MAC_PTR_HOST) {
        size_t need = host_fab_elems(c, -1, ng_rh) + host_fab_elems(c, -1, ng_phi);
        for (int d = 0; d < c->dm; ++d) need += host_fab_elems(c, d, ng_beta);
        if (alpha) need += host_fab_elems(c, -1, ng_alpha);
        rc = staging_reserve(c, need);
    }
    for (int d = 0; d < c->dm && !rc; ++d)
        rc = gather_faces(c, ptr_kind, beta + d * nb, ng_beta, d, c->u[d]);
    if (!rc) rc = gather_cells(c, ptr_kind, rh, ng_rh, 1, 0, c->rhs);
    if (!rc && alpha) rc = gather_cells(c, ptr_kind, alpha, ng_alpha, 1, 0, c->scratch);
    if (!rc) rc = gather_cells(c, ptr_kind, (const double* const*)phi, ng_phi, 1, 0, c->phin);
    if (!rc) {
        cudaEventRecord(c->ev[0], c->stream);
        rc = setup_fine_from_faces(c, c->u[0], c->u[1], c->dm == 3 ? c->u[2] : nullptr,
                                   alpha ? c->scratch : nullptr);
    }
    if (!rc) rc = setup_coarse_levels(c);
    if (!rc) rc = setup_rhs_from(c, c->rhs, c->phin);   // also moves phi into the level-0 layout
    int solve_rc = MAC_OK;
    if (!rc) {
        cudaEventRecord(c->ev[1], c->stream);
        solve_rc = run_solve(c, st);
        if (solve_rc != MAC_OK && solve_rc != MAC_ERR_NOT_CONVERGED) rc = solve_rc;
        cudaEventRecord(c->ev[2], c->stream);
    }
    if (!rc) rc = level0_to_natural(c, F.a64.phi, c->phin);
    if (!rc) rc = scatter_cells(c, ptr_kind, phi, ng_phi, c->phin);
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(c->xfer);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
            set_last_cuda_error(e, "cudaStreamSynchronize", __FILE__, __LINE__);
            rc = MAC_ERR_CUDA;
        } else {
            float a = 0.f, b = 0.f;
            cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
            cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
            st->setup_ms = a;
            st->solve_ms = b;
        }
    }
    if (!rc) rc = solve_rc;
    st->status = rc;
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    finish_stats(c, st);
    report(c, "mac_multigrid", st);
    return rc;
}

int mac_cell_to_edge(int nr, const double* s0_cell, double* s0_edge) {
    if (nr < 1 || !s0_cell || !s0_edge) return MAC_ERR_INVALID;
    for (int r = 0; r <= nr; ++r) {
        if (r == 0) {
            s0_edge[r] = s0_cell[0];
        } else if (r == 1) {
            s0_edge[r] = 0.5 * (s0_cell[0] + s0_cell[1 < nr ? 1 : 0]);
        } else if (r == nr) {
            s0_edge[r] = s0_cell[r - 1];
        } else if (r == nr - 1) {
            s0_edge[r] = 0.5 * (s0_cell[r] + s0_cell[r - 1]);
        } else {
            const double tmp = 7.0 / 12.0 * (s0_cell[r] + s0_cell[r - 1]) -
                               1.0 / 12.0 * (s0_cell[r + 1] + s0_cell[r - 2]);
            const double lo = s0_cell[r] < s0_cell[r - 1] ? s0_cell[r] : s0_cell[r - 1];
            const double hi = s0_cell[r] < s0_cell[r - 1] ? s0_cell[r - 1] : s0_cell[r];
            s0_edge[r] = tmp < lo ? lo : (tmp > hi ? hi : tmp);
        }
    }
    return MAC_OK;
}

}  // extern "C"
