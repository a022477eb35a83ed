// Finest-level FP32 kernels of the mixed-precision solve with the face coefficients computed on
// the fly from an FP32 copy of the density, instead of reading stored coefficient arrays:
//   beta'_f = fac_d[layer] / (rho_a + rho_b),   fac_d = beta0_f^p * 2 / h_d^2
// (the coefficient of Source/macproject.f90:698-738 times beta0 of :184-203, divided by h^2).
// A red/black half-sweep then reads the other colour's e and rho, its own r and rho and writes
// its own e: 10 bytes per cell of the level instead of 20 with stored FP32 coefficients.  Only the
// inner (FP32) V-cycle uses these; the FP64 refinement residual keeps the stored FP64 operator.
#include "mac_internal.cuh"
#include "mac_otf.cuh"

#include <algorithm>
#include <mutex>

namespace mac {
namespace {

constexpr int kB = 256;

template <int DM, bool SOR>
__global__ void __launch_bounds__(kB)
k_gsrb_otf(Dims d, OtfParams P, int colour, float* __restrict__ es, const float* __restrict__ eo,
           const float* __restrict__ rs, const float* __restrict__ rhos,
           const float* __restrict__ rhoo) {
    pdl_wait();
    pdl_trigger();
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (h >= d.hn0 || j >= d.n1) return;
    const int q = (j + d.n1 * k) * d.hn0 + h;
    const int i = 2 * h + ((colour + j + k) & 1);
    Nb nb;
    nbrs(d, colour, h, j, k, nb);
    float acc = rs[q], diag;
    otf_cell<DM>(P, nb, i, j, k, rhos[q], rhoo, eo, acc, diag);
    if (SOR) {
        const float old = es[q];
        es[q] = fmaf(P.omega, acc * rcp_approx(diag) - old, old);
    } else {
        es[q] = acc * rcp_approx(diag);
    }
}

// ---- staged 3-D half-sweep -------------------------------------------------------------------
// A block owns a tile of all hn0 colour-half columns x ty rows and marches through zc planes.
// Per plane, one thread issues bulk async copies (cp.async.bulk, completion counted on an
// mbarrier) of the other colour's e and rho on rows j0-1 .. j0+ty (wrapped) and the own colour's
// r and rho on rows j0 .. j0+ty-1 into a ring of kStages shared-memory stages, up to
// kStages - 1 planes ahead of the plane being updated.  Per plane, thread 0 waits on the
// mbarrier of the next plane and one block barrier publishes it to the other threads (they do
// not poll) and frees the stage read last for the next copy.  Each thread updates 4 consecutive
// own cells of one row (float4 reads of the stage); the other colour's centre row of planes
// k-1 / k / k+1 is carried in registers.  Arithmetic per cell is that of otf_cell, in the same
// order (the x-parity and the Dirichlet terms resolved at compile time).  Every wait is bounded
// (P.wait_ns of %globaltimer, mac_opts.wait_limit_s, one second by default); on expiry the block
// records the failure in P.err, waits (bounded by kDrainNs) for the copies it issued and leaves.  4 ring stages at 256^3 (ty = 8): 72 KB of
// shared memory and 80 registers a thread, 3 blocks per SM.
// Tunables of the staged half-sweep (compile-time; the defaults are the measured best at 256^3):
// cells of a tile, ring stages, and the resident blocks per SM its register budget is set for.
#ifndef MAC_OTF_TILE_CELLS
#define MAC_OTF_TILE_CELLS 1024
#endif
#ifndef MAC_OTF_STAGES
#define MAC_OTF_STAGES 4
#endif
#ifndef MAC_OTF_MIN_BLOCKS
#define MAC_OTF_MIN_BLOCKS 3
#endif
constexpr int kStages = MAC_OTF_STAGES;   // planes in the shared-memory ring
constexpr int kRStages = 3;         // the same for the staged restriction (one more array a plane)
constexpr int kCellsPerThread = 4;  // consecutive colour-half columns (one float4) per thread
// waits for copies a block has already seen arrive or that are draining after a failed wait
constexpr unsigned long long kDrainNs = 1000000000ull;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}
// try_wait with a suspend-time hint: the waiting thread sleeps (up to the hint) until the phase
// completes instead of spinning on issue slots its sub-partition's other warps need.
constexpr uint32_t kSuspendNs = 20000;
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(kSuspendNs)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Wait for phase `parity` of the mbarrier; false after about limit_ns without completion.
__device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned n = 1;; ++n) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((n & 63u) == 0 && global_ns() - t0 > limit_ns) return false;
    }
}

template <int V>
struct FV {
    float v[V];
};
template <int V>
__device__ __forceinline__ FV<V> ldv(const float* p) {
    FV<V> r;
    if constexpr (V == 4) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    } else {
        const float2 t = *reinterpret_cast<const float2*>(p);
        r.v[0] = t.x; r.v[1] = t.y;
    }
    return r;
}
template <int V>
__device__ __forceinline__ void stv(float* p, const float* v) {
    if constexpr (V == 4)
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    else
        *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
}

// Updates V consecutive own cells of one row (colour-half columns c0 .. c0+V-1) whose x-parity
// is SP (i = 2 (c0 + m) + SP); ex/rx = the other colour's value at the column just outside the
// group on the side SP selects (c0 - 1 for SP = 0, c0 + V for SP = 1).  fxl0 / fxhV: x factors
// of the group's outer low / high faces (zero on a non-periodic wall); wx0 / wxV / wmid: the
// Dirichlet diagonal factors of the first, last and inner cells (DIR only).
template <int V, int SP, bool DIR, bool RES = false, bool KEEP = false>
__device__ __forceinline__ void update_group(float ex, float rx, const FV<V>& Ec, const FV<V>& Rc,
                                             const FV<V>& Eb, const FV<V>& Rb, const FV<V>& Ea,
                                             const FV<V>& Ra, const FV<V>& Eym, const FV<V>& Rym,
                                             const FV<V>& Eyp, const FV<V>& Ryp, const FV<V>& Fo,
                                             const FV<V>& Ro, float fx, float fxl0, float fxhV,
                                             float fyl, float fyh, float fzl, float fzh,
                                             float wx0, float wxV, float wmid, float* out,
                                             const float* eown = nullptr, float* accv = nullptr,
                                             float* dgv = nullptr) {
#pragma unroll
    for (int m = 0; m < V; ++m) {
        const float rc = Ro.v[m];
        float el, rl, eh, rh, fl, fh;
        if (SP == 0) {
            el = m == 0 ? ex : Ec.v[m - 1];
            rl = m == 0 ? rx : Rc.v[m - 1];
            eh = Ec.v[m];
            rh = Rc.v[m];
            fl = m == 0 ? fxl0 : fx;
            fh = fx;
        } else {
            el = Ec.v[m];
            rl = Rc.v[m];
            eh = m == V - 1 ? ex : Ec.v[m + 1];
            rh = m == V - 1 ? rx : Rc.v[m + 1];
            fl = fx;
            fh = m == V - 1 ? fxhV : fx;
        }
        float acc = Fo.v[m];
        float b = fl * rcp_approx(rc + rl);
        acc = fmaf(b, el, acc);
        float dg = b;
        b = fh * rcp_approx(rc + rh);
        acc = fmaf(b, eh, acc);
        dg += b;
        b = fyl * rcp_approx(rc + Rym.v[m]);
        acc = fmaf(b, Eym.v[m], acc);
        dg += b;
        b = fyh * rcp_approx(rc + Ryp.v[m]);
        acc = fmaf(b, Eyp.v[m], acc);
        dg += b;
        b = fzl * rcp_approx(rc + Rb.v[m]);
        acc = fmaf(b, Eb.v[m], acc);
        dg += b;
        b = fzh * rcp_approx(rc + Ra.v[m]);
        acc = fmaf(b, Ea.v[m], acc);
        dg += b;
        if (DIR) {
            const float w = (SP == 0 && m == 0) ? wx0 : (SP == 1 && m == V - 1) ? wxV : wmid;
            dg += w * rcp_approx(rc);
        }
        // RES: the defect f - L e of the own cell instead of its Gauss-Seidel update; KEEP: also
        // hand back f + sum(arms) and the diagonal (the defect after an over-relaxed update)
        out[m] = RES ? fmaf(-dg, eown[m], acc) : acc * rcp_approx(dg);
        if (KEEP) {
            accv[m] = acc;
            dgv[m] = dg;
        }
    }
}

// DEF (with SOR): also write each updated cell's defect f - L e after its update to dout
// (indexed like es): after the over-relaxed half-sweep it is acc - diag e_new, no longer zero.
template <bool DIR, bool SOR, bool DEF = false>
__global__ void __launch_bounds__(MAC_OTF_TILE_CELLS / kCellsPerThread, MAC_OTF_MIN_BLOCKS)
k_gsrb_otf_staged(Dims d, OtfParams P, int colour, float* __restrict__ es,
                  const float* __restrict__ eo, const float* __restrict__ rs,
                  const float* __restrict__ rhos, const float* __restrict__ rhoo,
                  float* __restrict__ dout = nullptr) {
    constexpr int V = kCellsPerThread;
    extern __shared__ __align__(128) float sm[];
    __shared__ int abort_flag;
    const int hn0 = d.hn0, n1 = d.n1, n2 = d.n2, TY = P.ty;
    const int oth = (TY + 2) * hn0;    // floats of one other-colour array in a stage
    const int own = TY * hn0;          // floats of one own-colour array in a stage
    const int stage = 2 * oth + 2 * own;
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(sm + kStages * stage);
    const int j0 = blockIdx.x * TY;
    const int k0 = blockIdx.y * P.zc;
    const int kend = min(k0 + P.zc, n2);
    const int nq = kend - k0 + 2;      // planes k0-1 .. kend, local index q = p - (k0 - 1)
    const long plane = (long)n1 * hn0;
    const int t = threadIdx.x;
    __shared__ unsigned long long never_bar;   // fault injection: no copy ever completes it
    if (t == 0) {
        for (int q = 0; q < kStages; ++q) mbar_init(smem_addr(&bars[q]), 1);
        if (P.inject_expiry) mbar_init(smem_addr(&never_bar), 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // thread 0: copy plane q into stage q % kStages.  Part 1: the densities of both colours,
    // with the expected bytes of the whole stage; part 2: the other colour's e and the own
    // right-hand side.  The FP32 densities are written by the setup only, launches before any
    // half-sweep, so part 1 of the first planes goes out before the launch-dependency wait and
    // overlaps the end of the previous launch; the previous launch may have written part 2.
    auto issue_part = [&](int q, int part) {
        const int sidx = q % kStages;
        int p = k0 - 1 + q;
        p += (p < 0) ? n2 : 0;
        p -= (p >= n2) ? n2 : 0;
        float* st = sm + sidx * stage;
        const uint32_t bar = smem_addr(&bars[sidx]);
        if (part == 1) mbar_expect_tx(bar, (uint32_t)stage * 4u);
        const long pb = (long)p * plane;
        const float* rows = part == 1 ? rhoo : eo;
        float* dst = part == 1 ? st + oth : st;
        int slot = 0;
        while (slot < TY + 2) {
            int row = j0 - 1 + slot;
            row += (row < 0) ? n1 : 0;
            row -= (row >= n1) ? n1 : 0;
            const int len = min(TY + 2 - slot, n1 - row);
            const uint32_t bytes = (uint32_t)(len * hn0) * 4u;
            bulk_g2s(smem_addr(dst + slot * hn0), rows + pb + (long)row * hn0, bytes, bar);
            slot += len;
        }
        if (part == 1)
            bulk_g2s(smem_addr(st + 2 * oth + own), rhos + pb + (long)j0 * hn0,
                     (uint32_t)own * 4u, bar);
        else
            bulk_g2s(smem_addr(st + 2 * oth), rs + pb + (long)j0 * hn0, (uint32_t)own * 4u, bar);
    };
    // the refills: the whole stage, each row's e and density copies issued together
    auto issue = [&](int q) {
        const int sidx = q % kStages;
        int p = k0 - 1 + q;
        p += (p < 0) ? n2 : 0;
        p -= (p >= n2) ? n2 : 0;
        float* st = sm + sidx * stage;
        const uint32_t bar = smem_addr(&bars[sidx]);
        mbar_expect_tx(bar, (uint32_t)stage * 4u);
        const long pb = (long)p * plane;
        int slot = 0;
        while (slot < TY + 2) {
            int row = j0 - 1 + slot;
            row += (row < 0) ? n1 : 0;
            row -= (row >= n1) ? n1 : 0;
            const int len = min(TY + 2 - slot, n1 - row);
            const uint32_t bytes = (uint32_t)(len * hn0) * 4u;
            bulk_g2s(smem_addr(st + slot * hn0), eo + pb + (long)row * hn0, bytes, bar);
            bulk_g2s(smem_addr(st + oth + slot * hn0), rhoo + pb + (long)row * hn0, bytes, bar);
            slot += len;
        }
        bulk_g2s(smem_addr(st + 2 * oth), rs + pb + (long)j0 * hn0, (uint32_t)own * 4u, bar);
        bulk_g2s(smem_addr(st + 2 * oth + own), rhos + pb + (long)j0 * hn0, (uint32_t)own * 4u,
                 bar);
    };
    int issued = 0;      // planes issued so far (thread 0)
    int confirmed = 0;   // planes whose copies thread 0 has seen complete
    const int first = min(kStages, nq);
    if (t == 0)
        for (int q = 0; q < first; ++q) issue_part(q, 1);
    pdl_wait();
    pdl_trigger();
    if (t == 0) {
        for (; issued < first; ++issued) issue_part(issued, 2);
    }
    // thread 0 waits for plane q; the __syncthreads that follows every call publishes the
    // stage (and a failed wait) to the other threads, which do not poll the barrier
    auto wait_plane = [&](int q) {
        if (t != 0 || abort_flag) return;
        const bool ok = (P.inject_expiry && q == 0)
                            ? mbar_wait(smem_addr(&never_bar), 0u, P.wait_ns)
                            : mbar_wait(smem_addr(&bars[q % kStages]),
                                        (uint32_t)((q / kStages) & 1), P.wait_ns);
        if (ok) {
            confirmed = q + 1;
        } else {
            abort_flag = 1;
            atomicExch(P.err, 1);
        }
    };

    // this thread's V cells: row r of the tile, columns c0 .. c0+V-1
    const int idx = V * t;
    const int r = idx / hn0, c0 = idx - r * hn0;
    const int j = j0 + r;
    const int cm = (c0 == 0) ? hn0 - 1 : c0 - 1;          // column left of the group (wrapped)
    const int cp = (c0 + V == hn0) ? 0 : c0 + V;          // column right of the group
    const bool jl = j > 0 || P.per[1], jh = j < n1 - 1 || P.per[1];
    // non-periodic x walls: the low face of i = 0 (c0 == 0, m == 0, s == 0) and the high face of
    // i = n0 - 1 (c0 + V == hn0, m == V - 1, s == 1)
    const bool wlo = !P.per[0] && c0 == 0, whi = !P.per[0] && c0 + V == hn0;
    // Dirichlet walls touching the group: x low (first cell, s = 0), x high (last cell, s = 1),
    // y (every cell of the row)
    const bool dxl = P.dlo[0] && c0 == 0, dxh = P.dhi[0] && c0 + V == hn0;
    const bool dy = (j == 0 && P.dlo[1]) || (j == n1 - 1 && P.dhi[1]);
    const int st_n = n2 + 1;
    const int ctr = (r + 1) * hn0 + c0;                    // centre row in an other-colour array

    wait_plane(0);
    wait_plane(1);
    __syncthreads();
    FV<V> Eb = ldv<V>(sm + ctr), Rb = ldv<V>(sm + oth + ctr);
    FV<V> Ec = ldv<V>(sm + stage + ctr), Rc = ldv<V>(sm + stage + oth + ctr);
    // SOR: the own cells' old values, loaded one plane ahead so that their latency overlaps a
    // whole plane's work
    const float* eown = es + (long)j * hn0 + c0;
    FV<V> Enext;
    if (SOR) Enext = ldv<V>(eown + (long)k0 * plane);
    for (int k = k0; k < kend; ++k) {
        const int q = k - k0 + 1;
        FV<V> Eold;
        if (SOR) {
            Eold = Enext;
            if (k + 1 < kend) Enext = ldv<V>(eown + (long)(k + 1) * plane);
        }
        wait_plane(q + 1);
        // every thread is done with stage (q - 1) % kStages: refill it with plane q - 1 + kStages
        __syncthreads();
        if (abort_flag) break;
        if (t == 0 && issued < nq) issue(issued++);
        const float* sc = sm + (q % kStages) * stage;
        const float* su = sm + ((q + 1) % kStages) * stage;
        const FV<V> Ea = ldv<V>(su + ctr), Ra = ldv<V>(su + oth + ctr);
        const int s = (colour + j + k) & 1;
        const int cx = s ? cp : cm;
        const float ex = sc[(r + 1) * hn0 + cx], rx = sc[oth + (r + 1) * hn0 + cx];
        const FV<V> Eym = ldv<V>(sc + r * hn0 + c0), Rym = ldv<V>(sc + oth + r * hn0 + c0);
        const FV<V> Eyp = ldv<V>(sc + (r + 2) * hn0 + c0), Ryp = ldv<V>(sc + oth + (r + 2) * hn0 + c0);
        const FV<V> Fo = ldv<V>(sc + 2 * oth + r * hn0 + c0);
        const FV<V> Ro = ldv<V>(sc + 2 * oth + own + r * hn0 + c0);
        const float fx = P.fac[k], fy = P.fac[st_n + k];
        const float fyl = jl ? fy : 0.f, fyh = jh ? fy : 0.f;
        const float fzl = P.fac[2 * st_n + k], fzh = P.fac[3 * st_n + k];
        const float fxl0 = wlo ? 0.f : fx, fxhV = whi ? 0.f : fx;
        float out[V], accv[V], dgv[V];
        if (DIR) {
            const float wmid = P.fac[4 * st_n + k] + (dy ? fy : 0.f);
            const float wx0 = wmid + (dxl ? fx : 0.f), wxV = wmid + (dxh ? fx : 0.f);
            if (s)
                update_group<V, 1, true, false, DEF>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym, Eyp,
                                                     Ryp, Fo, Ro, fx, fxl0, fxhV, fyl, fyh, fzl,
                                                     fzh, wx0, wxV, wmid, out, nullptr, accv, dgv);
            else
                update_group<V, 0, true, false, DEF>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym, Eyp,
                                                     Ryp, Fo, Ro, fx, fxl0, fxhV, fyl, fyh, fzl,
                                                     fzh, wx0, wxV, wmid, out, nullptr, accv, dgv);
        } else if (s) {
            update_group<V, 1, false, false, DEF>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym, Eyp,
                                                  Ryp, Fo, Ro, fx, fxl0, fxhV, fyl, fyh, fzl, fzh,
                                                  0.f, 0.f, 0.f, out, nullptr, accv, dgv);
        } else {
            update_group<V, 0, false, false, DEF>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym, Eyp,
                                                  Ryp, Fo, Ro, fx, fxl0, fxhV, fyl, fyh, fzl, fzh,
                                                  0.f, 0.f, 0.f, out, nullptr, accv, dgv);
        }
        if (SOR) {
#pragma unroll
            for (int m = 0; m < V; ++m) out[m] = fmaf(P.omega, out[m] - Eold.v[m], Eold.v[m]);
        }
        const long cell = (long)k * plane + (long)j * hn0 + c0;
        stv<V>(es + cell, out);
        if (DEF) {
            float dv[V];
#pragma unroll
            for (int m = 0; m < V; ++m) dv[m] = fmaf(-dgv[m], out[m], accv[m]);
            stv<V>(dout + cell, dv);
        }
        Eb = Ec;
        Rb = Rc;
        Ec = Ea;
        Rc = Ra;
    }
    if (t == 0 && confirmed < issued) {
        // a wait gave up: leave no copy in flight into this block's shared memory (bounded)
        for (int q = confirmed; q < issued; ++q)
            mbar_wait(smem_addr(&bars[q % kStages]), (uint32_t)((q / kStages) & 1), kDrainNs);
    }
}

// Defect of the colour-0 cells of the finest FP32 level (after a colour-1 half-sweep the
// colour-1 defect vanishes) restricted into the coarse right-hand side, staged like
// k_gsrb_otf_staged: a block owns all colour-half columns of P.rty rows and marches through an
// even number of planes; the stage adds the own colour's e rows to the half-sweep's stage.  A
// thread forms the defects of its 4 cells (columns c0 .. c0+3 = coarse columns I), sums the two
// planes of a coarse plane in registers and the two rows of a coarse row through shared memory,
// then writes the 4 coarse values (two float2 per colour half of the coarse level) and zeroes the
// coarse correction there.  Same per-cell arithmetic as k_resid_restrict_otf; the eight children
// are summed as (plane pair per row) then (row pair).
// BLK: the colour-1 defects are not zero (an over-relaxed colour-1 half-sweep came last) and
// were written by that half-sweep into blk (colour-1 half indexing): each thread adds those of
// its row's colour-1 cells, the same colour-half columns, to its sums.
template <bool DIR, bool BLK = false>
__global__ void __launch_bounds__(256, 3)
k_resid_restrict_staged(Dims d, Dims C, OtfParams P, const float* __restrict__ eo,
                        const float* __restrict__ eown, const float* __restrict__ rs,
                        const float* __restrict__ rhos, const float* __restrict__ rhoo,
                        float* __restrict__ fc, float* __restrict__ ec,
                        const float* __restrict__ blk = nullptr) {
    constexpr int V = kCellsPerThread;
    constexpr int colour = 0;
    extern __shared__ __align__(128) float sm[];
    __shared__ int abort_flag;
    __shared__ __align__(16) float comb[256 * V];
    const int hn0 = d.hn0, n1 = d.n1, n2 = d.n2, TY = P.rty;
    const int oth = (TY + 2) * hn0;
    const int own = TY * hn0;
    const int stage = 2 * oth + 3 * own;
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(sm + kRStages * stage);
    const int j0 = blockIdx.x * TY;
    const int k0 = blockIdx.y * P.rzc;
    const int kend = min(k0 + P.rzc, n2);
    const int nq = kend - k0 + 2;
    const long plane = (long)n1 * hn0;
    const int t = threadIdx.x;
    __shared__ unsigned long long never_bar;   // fault injection: no copy ever completes it
    if (t == 0) {
        for (int q = 0; q < kRStages; ++q) mbar_init(smem_addr(&bars[q]), 1);
        if (P.inject_expiry) mbar_init(smem_addr(&never_bar), 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    pdl_wait();
    pdl_trigger();

    auto issue = [&](int q) {
        const int sidx = q % kRStages;
        int p = k0 - 1 + q;
        p += (p < 0) ? n2 : 0;
        p -= (p >= n2) ? n2 : 0;
        float* st = sm + sidx * stage;
        const uint32_t bar = smem_addr(&bars[sidx]);
        mbar_expect_tx(bar, (uint32_t)stage * 4u);
        const long pb = (long)p * plane;
        int slot = 0;
        while (slot < TY + 2) {
            int row = j0 - 1 + slot;
            row += (row < 0) ? n1 : 0;
            row -= (row >= n1) ? n1 : 0;
            const int len = min(TY + 2 - slot, n1 - row);
            const uint32_t bytes = (uint32_t)(len * hn0) * 4u;
            bulk_g2s(smem_addr(st + slot * hn0), eo + pb + (long)row * hn0, bytes, bar);
            bulk_g2s(smem_addr(st + oth + slot * hn0), rhoo + pb + (long)row * hn0, bytes, bar);
            slot += len;
        }
        const uint32_t ob = (uint32_t)own * 4u;
        bulk_g2s(smem_addr(st + 2 * oth), rs + pb + (long)j0 * hn0, ob, bar);
        bulk_g2s(smem_addr(st + 2 * oth + own), rhos + pb + (long)j0 * hn0, ob, bar);
        bulk_g2s(smem_addr(st + 2 * oth + 2 * own), eown + pb + (long)j0 * hn0, ob, bar);
    };
    int issued = 0, confirmed = 0;
    if (t == 0) {
        for (; issued < min(kRStages, nq); ++issued) issue(issued);
    }
    auto wait_plane = [&](int q) {
        if (t != 0 || abort_flag) return;
        const bool ok = (P.inject_expiry && q == 0)
                            ? mbar_wait(smem_addr(&never_bar), 0u, P.wait_ns)
                            : mbar_wait(smem_addr(&bars[q % kRStages]),
                                        (uint32_t)((q / kRStages) & 1), P.wait_ns);
        if (ok) {
            confirmed = q + 1;
        } else {
            abort_flag = 1;
            atomicExch(P.err, 1);
        }
    };

    const int idx = V * t;
    const int r = idx / hn0, c0 = idx - r * hn0;
    const int j = j0 + r;
    const int cm = (c0 == 0) ? hn0 - 1 : c0 - 1;
    const int cp = (c0 + V == hn0) ? 0 : c0 + V;
    const bool jl = j > 0 || P.per[1], jh = j < n1 - 1 || P.per[1];
    const bool wlo = !P.per[0] && c0 == 0, whi = !P.per[0] && c0 + V == hn0;
    const bool dxl = P.dlo[0] && c0 == 0, dxh = P.dhi[0] && c0 + V == hn0;
    const bool dy = (j == 0 && P.dlo[1]) || (j == n1 - 1 && P.dhi[1]);
    const int st_n = n2 + 1;
    const int ctr = (r + 1) * hn0 + c0;

    wait_plane(0);
    wait_plane(1);
    __syncthreads();
    FV<V> Eb = ldv<V>(sm + ctr), Rb = ldv<V>(sm + oth + ctr);
    FV<V> Ec = ldv<V>(sm + stage + ctr), Rc = ldv<V>(sm + stage + oth + ctr);
    float racc[V];
    for (int k = k0; k < kend; ++k) {
        const int q = k - k0 + 1;
        FV<V> Db;
        if (BLK) Db = ldv<V>(blk + (long)k * plane + (long)j * hn0 + c0);
        wait_plane(q + 1);
        __syncthreads();
        if (abort_flag) break;
        if (t == 0 && issued < nq) issue(issued++);
        const float* sc = sm + (q % kRStages) * stage;
        const float* su = sm + ((q + 1) % kRStages) * stage;
        const FV<V> Ea = ldv<V>(su + ctr), Ra = ldv<V>(su + oth + ctr);
        const int s = (colour + j + k) & 1;
        const int cx = s ? cp : cm;
        const float ex = sc[(r + 1) * hn0 + cx], rx = sc[oth + (r + 1) * hn0 + cx];
        const FV<V> Eym = ldv<V>(sc + r * hn0 + c0), Rym = ldv<V>(sc + oth + r * hn0 + c0);
        const FV<V> Eyp = ldv<V>(sc + (r + 2) * hn0 + c0);
        const FV<V> Ryp = ldv<V>(sc + oth + (r + 2) * hn0 + c0);
        const FV<V> Fo = ldv<V>(sc + 2 * oth + r * hn0 + c0);
        const FV<V> Ro = ldv<V>(sc + 2 * oth + own + r * hn0 + c0);
        const FV<V> Eown = ldv<V>(sc + 2 * oth + 2 * own + r * hn0 + c0);
        const float fx = P.fac[k], fy = P.fac[st_n + k];
        const float fyl = jl ? fy : 0.f, fyh = jh ? fy : 0.f;
        const float fzl = P.fac[2 * st_n + k], fzh = P.fac[3 * st_n + k];
        const float fxl0 = wlo ? 0.f : fx, fxhV = whi ? 0.f : fx;
        float res[V];
        if (DIR) {
            const float wmid = P.fac[4 * st_n + k] + (dy ? fy : 0.f);
            const float wx0 = wmid + (dxl ? fx : 0.f), wxV = wmid + (dxh ? fx : 0.f);
            if (s)
                update_group<V, 1, true, true>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym, Eyp, Ryp,
                                               Fo, Ro, fx, fxl0, fxhV, fyl, fyh, fzl, fzh, wx0,
                                               wxV, wmid, res, Eown.v);
            else
                update_group<V, 0, true, true>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym, Eyp, Ryp,
                                               Fo, Ro, fx, fxl0, fxhV, fyl, fyh, fzl, fzh, wx0,
                                               wxV, wmid, res, Eown.v);
        } else if (s) {
            update_group<V, 1, false, true>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym, Eyp, Ryp, Fo,
                                            Ro, fx, fxl0, fxhV, fyl, fyh, fzl, fzh, 0.f, 0.f, 0.f,
                                            res, Eown.v);
        } else {
            update_group<V, 0, false, true>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym, Eyp, Ryp, Fo,
                                            Ro, fx, fxl0, fxhV, fyl, fyh, fzl, fzh, 0.f, 0.f, 0.f,
                                            res, Eown.v);
        }
        if (BLK) {
#pragma unroll
            for (int m = 0; m < V; ++m) res[m] += Db.v[m];
        }
        if ((k & 1) == 0) {
#pragma unroll
            for (int m = 0; m < V; ++m) racc[m] = res[m];
        } else {
#pragma unroll
            for (int m = 0; m < V; ++m) racc[m] += res[m];
            // rows 2J (even r) and 2J+1 (odd r) of coarse row J: the odd row hands its sums over
            if (r & 1) *reinterpret_cast<float4*>(comb + V * t) = make_float4(racc[0], racc[1], racc[2], racc[3]);
            __syncthreads();
            if (!(r & 1)) {
                const float4 o = *reinterpret_cast<const float4*>(comb + V * (t + hn0 / V));
                const float v0 = (racc[0] + o.x) * 0.125f, v1 = (racc[1] + o.y) * 0.125f;
                const float v2 = (racc[2] + o.z) * 0.125f, v3 = (racc[3] + o.w) * 0.125f;
                const int J = j >> 1, K = k >> 1;
                const int pc = (c0 + J + K) & 1;   // coarse colour of I = c0 (and c0 + 2)
                const long base = (long)(J + C.n1 * K) * C.hn0 + (c0 >> 1);
                *reinterpret_cast<float2*>(fc + pc * C.half + base) = make_float2(v0, v2);
                *reinterpret_cast<float2*>(fc + (pc ^ 1) * C.half + base) = make_float2(v1, v3);
                *reinterpret_cast<float2*>(ec + pc * C.half + base) = make_float2(0.f, 0.f);
                *reinterpret_cast<float2*>(ec + (pc ^ 1) * C.half + base) = make_float2(0.f, 0.f);
            }
        }
        Eb = Ec;
        Rb = Rc;
        Ec = Ea;
        Rc = Ra;
    }
    if (t == 0 && confirmed < issued) {
        for (int q = confirmed; q < issued; ++q)
            mbar_wait(smem_addr(&bars[q % kRStages]), (uint32_t)((q / kRStages) & 1), kDrainNs);
    }
}

// ---- fused red + black sweep -----------------------------------------------------------------
// One whole sweep (colour 0, then colour 1 from the new colour-0 values) of the finest FP32
// level in one HBM pass, out of place: ein -> eout (both colours), so no block ever reads a value
// another block has already updated.  A block owns T rows of whole colour-half planes and a
// chunk of planes [k0, kend) and marches a wavefront up z: step s updates colour 0 on plane s
// (its T rows and one halo row on each side, which the colour-1 updates of its edge rows need;
// planes k0-1 and kend likewise) and colour 1 on plane s-1 from the new colour-0 values of planes
// s-2, s-1, s.  The shared-memory ring holds, per plane, only what other threads read: the old
// colour-1 e and rho on rows j0-2 .. j0+T+1 and the colour-0 rho on rows j0-1 .. j0+T, copied by
// bulk async copies; values of a thread's own row travel in registers along z, and the new
// colour-0 values of the last plane are exchanged through a double-buffered shared plane.  The
// per-cell arithmetic is update_group's, in the same order as the two half-sweeps, so the result
// is bitwise that of k_gsrb_otf_staged colour 0 then colour 1.  DEF: the colour-1 cells' defects
// after their update go to dout (colour-half indexing), as the DEF half-sweep writes them.
constexpr int kFMaxThreads = 320;   // (T + 2) rows x hn0 / 4 groups (two blocks an SM)

template <bool DIR, bool SOR, bool DEF>
__global__ void __launch_bounds__(kFMaxThreads, 2)
k_sweep_otf_fused(Dims d, OtfParams P, const float* __restrict__ ein, float* __restrict__ eout,
                  const float* __restrict__ rhs, float* __restrict__ dout) {
    constexpr int V = kCellsPerThread;
    extern __shared__ __align__(128) float sm[];
    __shared__ int abort_flag;
    __shared__ unsigned long long never_bar;   // fault injection: no copy ever completes it
    const int hn0 = d.hn0, n1 = d.n1, n2 = d.n2, T = P.fty, NS = P.fst;
    const long half = d.half;
    const int rE = T + 4, r0 = T + 2;                 // rows of the colour-1 / colour-0 arrays
    const int stage = (2 * rE + r0) * hn0;            // floats: e1, rho1, rho0
    float* nbuf = sm + NS * stage;                    // [2][T + 2][hn0] new colour-0 e
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(nbuf + 2 * r0 * hn0);
    const int j0 = blockIdx.x * T;
    const int k0 = blockIdx.y * P.fzc;
    const int kend = min(k0 + P.fzc, n2);
    const int nq = kend - k0 + 4;      // planes k0-2 .. kend+1, local index q = p - (k0 - 2)
    const long plane = (long)n1 * hn0;
    const int t = threadIdx.x;
    const float* e1in = ein + half;
    const float* rho0 = P.rho;
    const float* rho1 = P.rho + half;
    if (t == 0) {
        for (int q = 0; q < NS; ++q) mbar_init(smem_addr(&bars[q]), 1);
        if (P.inject_expiry) mbar_init(smem_addr(&never_bar), 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    pdl_wait();
    pdl_trigger();

    auto wrapk = [&](int p) { return p < 0 ? p + n2 : (p >= n2 ? p - n2 : p); };
    // thread 0: copy plane q into stage q % NS (rows wrapped; a tile row range may wrap around)
    auto copy_rows = [&](float* dst, const float* src, int first, int nrows, uint32_t bar) {
        int slot = 0;
        while (slot < nrows) {
            int row = first + slot;
            row += (row < 0) ? n1 : 0;
            row -= (row >= n1) ? n1 : 0;
            const int len = min(nrows - slot, n1 - row);
            bulk_g2s(smem_addr(dst + slot * hn0), src + (long)row * hn0,
                     (uint32_t)(len * hn0) * 4u, bar);
            slot += len;
        }
    };
    auto issue = [&](int q) {
        const int sidx = q % NS;
        const long pb = (long)wrapk(k0 - 2 + q) * plane;
        float* st = sm + sidx * stage;
        const uint32_t bar = smem_addr(&bars[sidx]);
        mbar_expect_tx(bar, (uint32_t)stage * 4u);
        copy_rows(st, e1in + pb, j0 - 2, rE, bar);
        copy_rows(st + rE * hn0, rho1 + pb, j0 - 2, rE, bar);
        copy_rows(st + 2 * rE * hn0, rho0 + pb, j0 - 1, r0, bar);
    };
    int issued = 0, confirmed = 0;
    if (t == 0) {
        for (; issued < min(NS, nq); ++issued) issue(issued);
    }
    auto wait_plane = [&](int q) {
        if (t != 0 || abort_flag) return;
        const bool ok = (P.inject_expiry && q == 0)
                            ? mbar_wait(smem_addr(&never_bar), 0u, P.wait_ns)
                            : mbar_wait(smem_addr(&bars[q % NS]), (uint32_t)((q / NS) & 1),
                                        P.wait_ns);
        if (ok) {
            confirmed = q + 1;
        } else {
            abort_flag = 1;
            atomicExch(P.err, 1);
        }
    };

    // this thread: row r of the tile (j = j0 - 1 + r, r = 0 and T + 1 are the halo rows that only
    // get colour-0 updates), columns c0 .. c0 + V - 1 of the colour halves
    const int G = hn0 / V;
    const int r = t / G, c0 = (t - r * G) * V;
    const bool own_row = r >= 1 && r <= T;
    int j = j0 - 1 + r;
    j += (j < 0) ? n1 : 0;
    j -= (j >= n1) ? n1 : 0;
    const int cm = (c0 == 0) ? hn0 - 1 : c0 - 1;
    const int cp = (c0 + V == hn0) ? 0 : c0 + V;
    const bool jl = j > 0 || P.per[1], jh = j < n1 - 1 || P.per[1];
    const bool wlo = !P.per[0] && c0 == 0, whi = !P.per[0] && c0 + V == hn0;
    const bool dxl = P.dlo[0] && c0 == 0, dxh = P.dhi[0] && c0 + V == hn0;
    const bool dy = (j == 0 && P.dlo[1]) || (j == n1 - 1 && P.dhi[1]);
    const int st_n = n2 + 1;
    const long rowoff = (long)j * hn0 + c0;
    // shared-memory offsets of this thread's columns: row r + 1 of the colour-1 arrays, row r of
    // the colour-0 ones
    const int o1 = (r + 1) * hn0 + c0, o0 = r * hn0 + c0;

    // factors of plane k, and the update of one group of the given colour
    auto group = [&](int colour, int k, float ex, float rx, const FV<V>& Ec, const FV<V>& Rc,
                     const FV<V>& Eb, const FV<V>& Rb, const FV<V>& Ea, const FV<V>& Ra,
                     const FV<V>& Eym, const FV<V>& Rym, const FV<V>& Eyp, const FV<V>& Ryp,
                     const FV<V>& Fo, const FV<V>& Ro, float* out, float* accv, float* dgv) {
        const int s = (colour + j + k) & 1;
        const float fx = P.fac[k], fy = P.fac[st_n + k];
        const float fyl = jl ? fy : 0.f, fyh = jh ? fy : 0.f;
        const float fzl = P.fac[2 * st_n + k], fzh = P.fac[3 * st_n + k];
        const float fxl0 = wlo ? 0.f : fx, fxhV = whi ? 0.f : fx;
        if (DIR) {
            const float wmid = P.fac[4 * st_n + k] + (dy ? fy : 0.f);
            const float wx0 = wmid + (dxl ? fx : 0.f), wxV = wmid + (dxh ? fx : 0.f);
            if (s)
                update_group<V, 1, true, false, true>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym,
                                                      Eyp, Ryp, Fo, Ro, fx, fxl0, fxhV, fyl, fyh,
                                                      fzl, fzh, wx0, wxV, wmid, out, nullptr,
                                                      accv, dgv);
            else
                update_group<V, 0, true, false, true>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym,
                                                      Eyp, Ryp, Fo, Ro, fx, fxl0, fxhV, fyl, fyh,
                                                      fzl, fzh, wx0, wxV, wmid, out, nullptr,
                                                      accv, dgv);
        } else if (s) {
            update_group<V, 1, false, false, true>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym, Eyp,
                                                   Ryp, Fo, Ro, fx, fxl0, fxhV, fyl, fyh, fzl,
                                                   fzh, 0.f, 0.f, 0.f, out, nullptr, accv, dgv);
        } else {
            update_group<V, 0, false, false, true>(ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym, Eyp,
                                                   Ryp, Fo, Ro, fx, fxl0, fxhV, fyl, fyh, fzl,
                                                   fzh, 0.f, 0.f, 0.f, out, nullptr, accv, dgv);
        }
        return s;
    };

    // Per step s the stages of planes s - 1, s and s + 1 are resident: the old colour-1 values of
    // the own row along z are read from them.  Registers carry only what no stage holds any more
    // (colour-0 rho and new e of plane s - 2, for the colour-1 update of plane s - 1) and the own
    // cells' f and old e (plain loads, issued one step ahead).
    //   f0c/e0c: colour-0 f and old e of plane s; f1c: colour-1 f of plane s - 1 (own rows)
    FV<V> r0m2, n0m2, f0c, e0c, f1c, f0n, e0n, f1n;
#pragma unroll
    for (int m = 0; m < V; ++m) {
        r0m2.v[m] = n0m2.v[m] = 0.f;
        e0c.v[m] = e0n.v[m] = f1c.v[m] = f1n.v[m] = 0.f;
    }
    // colour-0 f and old e of plane p, colour-1 f of plane p - 1 (the plane colour 1 is updated
    // on in the same step as colour 0 on plane p)
    auto load_own = [&](int p, FV<V>& f0x, FV<V>& e0x, FV<V>& f1x) {
        const long base = (long)wrapk(p) * plane + rowoff;
        f0x = ldv<V>(rhs + base);
        if (SOR) e0x = ldv<V>(ein + base);
        if (own_row) f1x = ldv<V>(rhs + half + (long)wrapk(p - 1) * plane + rowoff);
    };
    load_own(k0 - 1, f0c, e0c, f1c);   // (f1 of plane k0 - 2 is never used)

    wait_plane(0);
    wait_plane(1);
    for (int s = k0 - 1; s <= kend; ++s) {
        const int q = s - k0 + 2;           // local index of plane s
        wait_plane(q + 1);
        __syncthreads();                    // plane q + 1 landed; nbuf of plane s - 1 complete
        if (abort_flag) break;
        if (t == 0 && q >= 2 && issued < nq) issue(issued++);   // the slot of plane q - 2 is free
        // the next plane's own values: their DRAM latency overlaps this step
        if (s + 1 <= kend) load_own(s + 1, f0n, e0n, f1n);
        const int ks = wrapk(s);
        const float* sc = sm + (q % NS) * stage;              // plane s
        const float* su = sm + ((q + 1) % NS) * stage;        // plane s + 1
        const float* sd = sm + ((q + NS - 1) % NS) * stage;   // plane s - 1
        const float* nb = nbuf + ((q - 1) & 1) * r0 * hn0;    // new colour 0, plane s - 1
        const FV<V> r0c = ldv<V>(sc + 2 * rE * hn0 + o0);    // colour-0 rho, planes s, s - 1
        const FV<V> r0m = ldv<V>(sd + 2 * rE * hn0 + o0);
        const FV<V> n0m = ldv<V>(nb + o0);

        // ---- colour 0 on plane s (all T + 2 rows)
        FV<V> n0c;
        {
            const int sp = (j + ks) & 1;
            const int cx = sp ? cp : cm;
            const float ex = sc[o1 - c0 + cx], rx = sc[rE * hn0 + o1 - c0 + cx];
            const FV<V> Ec = ldv<V>(sc + o1), Rc = ldv<V>(sc + rE * hn0 + o1);
            const FV<V> Eb = ldv<V>(sd + o1), Rb = ldv<V>(sd + rE * hn0 + o1);
            const FV<V> Ea = ldv<V>(su + o1), Ra = ldv<V>(su + rE * hn0 + o1);
            const FV<V> Eym = ldv<V>(sc + o1 - hn0), Rym = ldv<V>(sc + rE * hn0 + o1 - hn0);
            const FV<V> Eyp = ldv<V>(sc + o1 + hn0), Ryp = ldv<V>(sc + rE * hn0 + o1 + hn0);
            float out[V], accv[V], dgv[V];
            group(0, ks, ex, rx, Ec, Rc, Eb, Rb, Ea, Ra, Eym, Rym, Eyp, Ryp, f0c, r0c, out, accv,
                  dgv);
            if (SOR) {
#pragma unroll
                for (int m = 0; m < V; ++m) out[m] = fmaf(P.omega, out[m] - e0c.v[m], e0c.v[m]);
            }
#pragma unroll
            for (int m = 0; m < V; ++m) n0c.v[m] = out[m];
            stv<V>(nbuf + (q & 1) * r0 * hn0 + o0, out);
            if (own_row && s >= k0 && s < kend) stv<V>(eout + (long)ks * plane + rowoff, out);
        }
        // ---- colour 1 on plane s - 1 (own rows), from the new colour-0 values
        if (s >= k0 + 1 && own_row) {
            const int km = wrapk(s - 1);
            const float* rb = sd + 2 * rE * hn0;                 // colour-0 rho, plane s - 1
            const int sp = (1 + j + km) & 1;
            const int cx = sp ? cp : cm;
            const float ex = nb[o0 - c0 + cx], rx = rb[o0 - c0 + cx];
            const FV<V> Eym = ldv<V>(nb + o0 - hn0), Rym = ldv<V>(rb + o0 - hn0);
            const FV<V> Eyp = ldv<V>(nb + o0 + hn0), Ryp = ldv<V>(rb + o0 + hn0);
            const FV<V> Ro = ldv<V>(sd + rE * hn0 + o1);        // own rho, plane s - 1
            float out[V], accv[V], dgv[V];
            group(1, km, ex, rx, n0m, r0m, n0m2, r0m2, n0c, r0c, Eym, Rym, Eyp, Ryp, f1c, Ro,
                  out, accv, dgv);
            if (SOR) {
                const FV<V> Eold = ldv<V>(sd + o1);              // own old e, plane s - 1
#pragma unroll
                for (int m = 0; m < V; ++m) out[m] = fmaf(P.omega, out[m] - Eold.v[m], Eold.v[m]);
            }
            const long cell = (long)km * plane + rowoff;
            stv<V>(eout + half + cell, out);
            if (DEF) {
                float dv[V];
#pragma unroll
                for (int m = 0; m < V; ++m) dv[m] = fmaf(-dgv[m], out[m], accv[m]);
                stv<V>(dout + cell, dv);
            }
        }
        r0m2 = r0m;
        n0m2 = n0m;
        f0c = f0n;
        e0c = e0n;
        f1c = f1n;
    }
    if (t == 0 && confirmed < issued) {
        // a wait gave up: leave no copy in flight into this block's shared memory (bounded)
        for (int q = confirmed; q < issued; ++q)
            mbar_wait(smem_addr(&bars[q % NS]), (uint32_t)((q / NS) & 1), kDrainNs);
    }
}

template <int DM, bool RED_ONLY>
__global__ void __launch_bounds__(kB)
k_resid_restrict_otf(Dims F, Dims C, OtfParams P, const float* __restrict__ e,
                     const float* __restrict__ r, float* __restrict__ fc, float* __restrict__ ec) {
    pdl_wait();
    pdl_trigger();
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int K = blockIdx.z;
    if (I >= C.n0 || J >= C.n1) return;
    const int rz = DM == 3 ? 2 : 1;
    float sum = 0.f;
#pragma unroll
    for (int b = 0; b < rz; ++b) {
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            const int j = 2 * J + a;
            const int k = DM == 3 ? 2 * K + b : K;
#pragma unroll
            for (int colour = 0; colour < (RED_ONLY ? 1 : 2); ++colour) {
                const int off = colour * F.half, oth = (colour ^ 1) * F.half;
                const int i = 2 * I + ((colour + j + k) & 1);
                Nb nb;
                nbrs(F, colour, I, j, k, nb);
                const int me = (j + F.n1 * k) * F.hn0 + I;
                float acc = r[off + me], diag;
                otf_cell<DM>(P, nb, i, j, k, P.rho[off + me], P.rho + oth, e + oth, acc, diag);
                sum += fmaf(-diag, e[off + me], acc);
            }
        }
    }
    int ci;
    if (C.split)
        ci = ((I + J + K) & 1) * C.half + (J + C.n1 * K) * C.hn0 + (I >> 1);
    else
        ci = I + C.n0 * (J + C.n1 * K);
    fc[ci] = sum * (DM == 3 ? 0.125f : 0.25f);
    ec[ci] = 0.f;   // the coarse correction starts from zero (no separate memset in the chain)
}

}  // namespace

void launch_gsrb_otf(const Dims& d, const OtfParams& P, int colour, float* e, const float* r,
                     cudaStream_t s, float* dout) {
    const int own = colour * d.half, oth = (colour ^ 1) * d.half;
    const Grid3 g = grid3(d.hn0, d.n1, d.n2);
    const bool sor = P.omega != 1.f;
    if (P.dm == 3 && P.ty > 0) {
        const dim3 grid(d.n1 / P.ty, P.nz);
        const int nt = P.ty * d.hn0 / kCellsPerThread;
        if (sor && dout) {
            auto kern = P.has_dir ? k_gsrb_otf_staged<true, true, true>
                                  : k_gsrb_otf_staged<false, true, true>;
            launch_chain(kern, grid, dim3(nt), (size_t)P.smem, s, d, P, colour, e + own,
                         (const float*)(e + oth), r + own, P.rho + own, P.rho + oth, dout);
            return;
        }
        auto kern = P.has_dir ? (sor ? k_gsrb_otf_staged<true, true> : k_gsrb_otf_staged<true, false>)
                              : (sor ? k_gsrb_otf_staged<false, true> : k_gsrb_otf_staged<false, false>);
        launch_chain(kern, grid, dim3(nt), (size_t)P.smem, s, d, P, colour, e + own,
                     (const float*)(e + oth), r + own, P.rho + own, P.rho + oth, (float*)nullptr);
    } else if (P.dm == 3) {
        auto kern = sor ? k_gsrb_otf<3, true> : k_gsrb_otf<3, false>;
        launch_chain(kern, g.grid, g.block, 0, s, d, P, colour, e + own, (const float*)(e + oth),
                     r + own, P.rho + own, P.rho + oth);
    } else {
        auto kern = sor ? k_gsrb_otf<2, true> : k_gsrb_otf<2, false>;
        launch_chain(kern, g.grid, g.block, 0, s, d, P, colour, e + own, (const float*)(e + oth),
                     r + own, P.rho + own, P.rho + oth);
    }
}

// Tile plan of the fused sweep: T = the largest divisor of n1 with (T + 2) * hn0 / 4 <= 320
// threads and T >= 4; the most ring stages (5, else 4) with which two blocks fit
// on an SM; chunks of planes so that the blocks fill the resident slots of every SM once.  Sets
// fty = 0 where the fused sweep does not apply.
void plan_fused_tile(const Dims& d, int sms, OtfParams& P) {
    static std::mutex mu;
    static int fsmem_set = 0;
    P.fty = P.fzc = P.fnz = P.fst = P.fsmem = P.fthreads = 0;
    const int G = d.hn0 / kCellsPerThread;
    int T = 0;
    for (int cand = d.n1; cand >= 4; --cand) {
        if (d.n1 % cand || (cand + 2) * G > kFMaxThreads) continue;
        T = cand;
        break;
    }
    if (T == 0 || d.n2 < 2) return;
    const int stage = (2 * (T + 4) + (T + 2)) * d.hn0;
    const int extra = 2 * (T + 2) * d.hn0;
    int NS = 5;
    int smem = (NS * stage + extra) * 4 + NS * 8;
    if (2 * smem > 220 * 1024) {
        NS = 4;
        smem = (NS * stage + extra) * 4 + NS * 8;
    }
    if (smem > 200 * 1024) return;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (smem > fsmem_set) {
            bool ok = true;
            auto setmax = [&](auto kern) {
                ok = ok && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                smem) == cudaSuccess;
            };
            setmax(k_sweep_otf_fused<false, false, false>);
            setmax(k_sweep_otf_fused<true, false, false>);
            setmax(k_sweep_otf_fused<false, true, false>);
            setmax(k_sweep_otf_fused<true, true, false>);
            setmax(k_sweep_otf_fused<false, true, true>);
            setmax(k_sweep_otf_fused<true, true, true>);
            setmax(k_sweep_otf_fused<false, false, true>);
            setmax(k_sweep_otf_fused<true, false, true>);
            if (!ok) {
                cudaGetLastError();
                return;
            }
            fsmem_set = smem;
        }
    }
    const int nt = (T + 2) * G;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep_otf_fused<false, true, false>,
                                                      nt, smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return;
    }
    const int tiles = d.n1 / T;
    long chunks = ((long)sms * per_sm) / tiles;
    if (chunks < 1) chunks = 1;
    int zc = ceil_div(d.n2, (int)std::min<long>(chunks, d.n2));
    if (zc < 4) zc = std::min(4, d.n2);
    P.fty = T;
    P.fzc = zc;
    P.fnz = ceil_div(d.n2, zc);
    P.fst = NS;
    P.fsmem = smem;
    P.fthreads = nt;
}

// Tile plan of the staged half-sweep: ty = the largest power of two with ty * hn0 <= 1024 cells
// that divides n1 (one float4 group of 4 cells per thread, at most 256 threads); whole rows of
// 16-byte multiples (hn0 % 4 == 0); chunks of planes so that the blocks fill the resident slots
// of every SM once.  Sets ty = 0 where the staged kernel does not apply.
void plan_otf_tile(const Dims& d, int dm, int sms, OtfParams& P) {
    static std::mutex mu;
    static int smem_set = 0;
    P.ty = P.zc = P.nz = P.smem = 0;
    P.rty = P.rzc = P.rnz = P.rsmem = 0;
    if (dm != 3 || !d.split || d.hn0 % 4 || d.hn0 > 1024 || d.n2 < 2) return;
    int ty = 1;
    while (2 * ty * d.hn0 <= MAC_OTF_TILE_CELLS && d.n1 % (2 * ty) == 0) ty *= 2;
    const int nt = ty * d.hn0 / kCellsPerThread;
    if (nt < 32 || nt % 32) return;
    const int stage = (4 * ty + 4) * d.hn0;
    const int smem = kStages * stage * 4 + kStages * 8;
    if (smem > 200 * 1024) return;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (smem > smem_set) {
            if (cudaFuncSetAttribute(k_gsrb_otf_staged<false, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_gsrb_otf_staged<true, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_gsrb_otf_staged<false, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_gsrb_otf_staged<true, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_gsrb_otf_staged<false, true, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_gsrb_otf_staged<true, true, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
                    cudaSuccess) {
                cudaGetLastError();
                return;
            }
            smem_set = smem;
        }
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gsrb_otf_staged<false, false>, nt,
                                                      smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return;
    }
    const long tiles = d.n1 / ty;
    long chunks = ((long)sms * per_sm) / tiles;
    if (chunks < 1) chunks = 1;
    int zc = ceil_div(d.n2, (int)std::min<long>(chunks, d.n2));
    if (zc < 4) zc = std::min(4, d.n2);
    P.ty = ty;
    P.zc = zc;
    P.nz = ceil_div(d.n2, zc);
    P.smem = smem;
    // staged defect + restriction: the same tiles, one more own-colour array in the stage, plane
    // chunks of even length (a coarse plane is two fine planes)
    static int rsmem_set = 0;
    const int rstage = (2 * (ty + 2) + 3 * ty) * d.hn0;
    const int rsmem = kRStages * rstage * 4 + kRStages * 8;
    if (ty % 2 || d.n2 % 2 || rsmem > 200 * 1024) return;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (rsmem > rsmem_set) {
            if (cudaFuncSetAttribute(k_resid_restrict_staged<false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, rsmem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_resid_restrict_staged<true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, rsmem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_resid_restrict_staged<false, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, rsmem) !=
                    cudaSuccess ||
                cudaFuncSetAttribute(k_resid_restrict_staged<true, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, rsmem) !=
                    cudaSuccess) {
                cudaGetLastError();
                return;
            }
            rsmem_set = rsmem;
        }
    }
    int rper_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rper_sm, k_resid_restrict_staged<false>,
                                                      nt, rsmem) != cudaSuccess ||
        rper_sm < 1) {
        cudaGetLastError();
        return;
    }
    long rchunks = ((long)sms * rper_sm) / tiles;
    if (rchunks < 1) rchunks = 1;
    int rzc = ceil_div(d.n2, (int)std::min<long>(rchunks, d.n2 / 2));
    rzc += rzc & 1;
    if (rzc < 4) rzc = std::min(4, d.n2);
    P.rty = ty;
    P.rzc = rzc;
    P.rnz = ceil_div(d.n2, rzc);
    P.rsmem = rsmem;
    plan_fused_tile(d, sms, P);
}

void launch_sweep_otf_fused(const Dims& d, const OtfParams& P, const float* ein, float* eout,
                            const float* r, cudaStream_t s, float* dout) {
    const dim3 grid(d.n1 / P.fty, P.fnz);
    const bool sor = P.omega != 1.f;
    auto kern = P.has_dir
                    ? (sor ? (dout ? k_sweep_otf_fused<true, true, true> : k_sweep_otf_fused<true, true, false>)
                           : (dout ? k_sweep_otf_fused<true, false, true> : k_sweep_otf_fused<true, false, false>))
                    : (sor ? (dout ? k_sweep_otf_fused<false, true, true> : k_sweep_otf_fused<false, true, false>)
                           : (dout ? k_sweep_otf_fused<false, false, true> : k_sweep_otf_fused<false, false, false>));
    launch_chain(kern, grid, dim3(P.fthreads), (size_t)P.fsmem, s, d, P, ein, eout, r, dout);
}

void launch_resid_restrict_otf(const Dims& fine, const Dims& coarse, const OtfParams& P,
                               const float* e, const float* r, float* fc, float* ec,
                               bool red_only, cudaStream_t s, const float* blk) {
    if (P.dm == 3 && P.rty > 0 && (red_only || blk) && coarse.split) {
        // colour 0 is "own": its e, f and rho; colour 1 the other colour's e and rho (and, after
        // an over-relaxed colour-1 half-sweep, its defects in blk)
        const dim3 grid(fine.n1 / P.rty, P.rnz);
        const int nt = P.rty * fine.hn0 / kCellsPerThread;
        const float* eo = e + fine.half;
        const float* rhoo = P.rho + fine.half;
        auto kern = red_only ? (P.has_dir ? k_resid_restrict_staged<true>
                                          : k_resid_restrict_staged<false>)
                             : (P.has_dir ? k_resid_restrict_staged<true, true>
                                          : k_resid_restrict_staged<false, true>);
        launch_chain(kern, grid, dim3(nt), (size_t)P.rsmem, s, fine, coarse, P, eo, e, r,
                     (const float*)P.rho, rhoo, fc, ec, red_only ? (const float*)nullptr : blk);
        return;
    }
    const Grid3 g = grid3(coarse.n0, coarse.n1, coarse.n2);
    if (P.dm == 3) {
        if (red_only)
            launch_chain(k_resid_restrict_otf<3, true>, g.grid, g.block, 0, s, fine, coarse, P, e, r,
                       fc, ec);
        else
            launch_chain(k_resid_restrict_otf<3, false>, g.grid, g.block, 0, s, fine, coarse, P, e,
                       r, fc, ec);
    } else {
        if (red_only)
            launch_chain(k_resid_restrict_otf<2, true>, g.grid, g.block, 0, s, fine, coarse, P, e, r,
                       fc, ec);
        else
            launch_chain(k_resid_restrict_otf<2, false>, g.grid, g.block, 0, s, fine, coarse, P, e,
                       r, fc, ec);
    }
}

}  // namespace mac
