// Multi-level (AMR) MAC projection: the composite discretisation cell by cell, and the
// multi-level cycle and projection steps written once against an executor.
//
// MAESTRO's macproject with nlevs > 1 (Source/macproject.f90:51-328) hands FBoxLib's composite
// solve ml_cc_solve a hierarchy of levels with refinement ratio 2 (Source/mac_multigrid.f90:56).
// Level l (n0 << l cells per active direction) is stored as arrays over its array box -- the
// bounding box of its boxes grown by one cell (level_box; level 0: the whole domain) -- in
// natural layout (i - lo0) + ext0 ((j - lo1) + ext1 (k - lo2)), with a byte mask: kIn for the
// cells of the level's boxes, kCov for the cells under the next finer level.  Valid cells (kIn
// without kCov) carry the composite unknowns; covered cells hold the mean of their children.
//
// Composite operator (the form FBoxLib describes in Docs/mg/mg.tex:124-155, stencil_order = 2):
//   * fine arms beta_f (u_c - u_nb) / h^2; across a coarse-fine face the neighbour is the ghost
//     u_c / 3 + 2/3 u_crse, the line through the first fine cell and the coarse value at the
//     centre of the coarse cell across the face; u_crse is that coarse cell corrected along each
//     tangential direction by the quadratic through its tangential neighbours at the ghost's
//     offset +-1/4 (one-sided linear at a non-periodic domain face);
//   * a valid coarse cell next to a covered one takes, for that face, the mean of the 2^(dm-1)
//     fine fluxes beta_f (ghost - u_fine) / h_fine instead of its own flux (reflux);
//   * physical faces: Neumann dropped, periodic wrapped, Dirichlet with the ghost -u_c.
//
// The per-cell functions below are plain C++ (host and device); mac_amr.cu launches them as
// CUDA kernels.  `amr_solve` / `amr_project` sequence a multi-level V-cycle and the projection
// steps through an executor `E` that owns the level arrays and applies the cell functions over
// a level (see GpuExec in mac_amr.cu).
#pragma once

#include <cmath>
#include <cstdint>
#include <type_traits>

#if defined(__CUDACC__)
#define AMR_HD __host__ __device__
#else
#define AMR_HD
#endif
#if defined(__CUDA_ARCH__)
#define AMR_UNROLL _Pragma("unroll")
#else
#define AMR_UNROLL
#endif

namespace mac {
namespace amr {

constexpr int kMaxLevels = 8;
constexpr unsigned char kIn = 1;
constexpr unsigned char kCov = 2;

struct Geo {
    int dm;
    int per[3];          // periodic direction
    int dlo[3], dhi[3];  // Dirichlet (outflow) domain faces
    int va;              // vertical direction (planar beta0 index): dm - 1
};

// A level with its face coefficients in precision T (FP64; FP32 for the inner cycles of the
// mixed-precision solve).
template <typename T>
struct LevT {
    int n[3];                  // level-domain cells (1 along inactive directions)
    int lo[3], ext[3];         // the array box: cells lo .. lo + ext - 1 of the level domain
    double h[3];
    double ih[3], ih2[3];      // 1 / h and 1 / h^2 (set with h by set_spacing: no division in
                               // the cell functions, FP64 division being slow on the GPU)
    const unsigned char* mask; // kIn / kCov per cell of the box
    const T* b[3];             // face coefficients over the box (ext[d] + 1 faces along d)
};
using Lev = LevT<double>;

template <typename T>
inline void set_spacing(LevT<T>& L, int d, double h) {
    L.h[d] = h;
    L.ih[d] = 1.0 / h;
    L.ih2[d] = 1.0 / (h * h);
}

// Array box of a level: the bounding box [rlo, rhi] of its cells grown by one cell and clipped
// to the domain; a periodic direction whose grown box would cross the domain face takes the
// whole extent (neighbours across the face are then in the box).  Level 0: the domain.
inline void level_box(int dm, const int n[3], const int per[3], const int rlo[3],
                      const int rhi[3], int lo[3], int ext[3]) {
    for (int d = 0; d < 3; ++d) {
        if (d >= dm) {
            lo[d] = 0;
            ext[d] = 1;
            continue;
        }
        int a = rlo[d] - 1, b = rhi[d] + 1;
        if (per[d] && (a < 0 || b > n[d] - 1)) {
            a = 0;
            b = n[d] - 1;
        }
        a = a < 0 ? 0 : a;
        b = b > n[d] - 1 ? n[d] - 1 : b;
        lo[d] = a;
        ext[d] = b - a + 1;
    }
}

// Index of cell / face (i, j, k) of the level domain in the box arrays (the caller keeps it in
// the box).
template <typename T>
AMR_HD inline long cix(const LevT<T>& L, int i, int j, int k) {
    return (long)(i - L.lo[0]) + (long)L.ext[0] * ((long)(j - L.lo[1]) + (long)L.ext[1] * (k - L.lo[2]));
}
template <typename T>
AMR_HD inline long fix(const LevT<T>& L, int d, int i, int j, int k) {
    const long m0 = L.ext[0] + (d == 0), m1 = L.ext[1] + (d == 1);
    return (long)(i - L.lo[0]) + m0 * ((long)(j - L.lo[1]) + m1 * (k - L.lo[2]));
}
template <typename T>
AMR_HD inline long nfaces(const LevT<T>& L, int d) {
    return (long)(L.ext[0] + (d == 0)) * (L.ext[1] + (d == 1)) * (L.ext[2] + (d == 2));
}
template <typename T>
AMR_HD inline long ncells(const LevT<T>& L) { return (long)L.ext[0] * L.ext[1] * L.ext[2]; }
template <typename T>
AMR_HD inline bool inside(const LevT<T>& L, const int c[3]) {
    AMR_UNROLL
    for (int d = 0; d < 3; ++d)
        if (c[d] < L.lo[d] || c[d] >= L.lo[d] + L.ext[d]) return false;
    return true;
}
template <typename T>
AMR_HD inline bool inside_face(const LevT<T>& L, int dir, const int f[3]) {
    for (int d = 0; d < 3; ++d)
        if (f[d] < L.lo[d] || f[d] >= L.lo[d] + L.ext[d] + (d == dir)) return false;
    return true;
}

// Index q along d wrapped into the level domain; -1 beyond a non-periodic domain face.
template <typename T>
AMR_HD inline int wrap(const Geo& G, const LevT<T>& L, int d, int q) {
    const int n = L.n[d];
    if (q < 0) return G.per[d] ? q + n : -1;
    if (q >= n) return G.per[d] ? q - n : -1;
    return q;
}
template <typename T>
AMR_HD inline bool in_region(const LevT<T>& L, long c) { return (L.mask[c] & kIn) != 0; }
template <typename T>
AMR_HD inline bool is_valid(const LevT<T>& L, long c) { return (L.mask[c] & (kIn | kCov)) == kIn; }

template <typename T>
AMR_HD inline T face_b(const LevT<T>& L, int d, const int c[3], int s) {
    int f[3] = {c[0], c[1], c[2]};
    if (s > 0) f[d] += 1;
    return L.b[d][fix(L, d, f[0], f[1], f[2])];
}

// Coarse value (level C, array cu) at the fine ghost cell q seen across a face normal to d.
template <typename T>
AMR_HD inline T coarse_at_ghost(const Geo& G, const LevT<T>& C, const int q[3], int d,
                                const T* cu) {
    int c[3];
    AMR_UNROLL
    for (int e = 0; e < 3; ++e) c[e] = e < G.dm ? q[e] >> 1 : q[e];
    const T v0 = cu[cix(C, c[0], c[1], c[2])];
    T v = v0;
    AMR_UNROLL
    for (int t = 0; t < 3; ++t) {
        if (t >= G.dm) break;
        if (t == d) continue;
        const T del = (q[t] & 1) ? (T)0.25 : (T)-0.25;
        int m[3] = {c[0], c[1], c[2]}, p[3] = {c[0], c[1], c[2]};
        m[t] = wrap(G, C, t, c[t] - 1);
        p[t] = wrap(G, C, t, c[t] + 1);
        const bool hm = m[t] >= 0, hp = p[t] >= 0;
        const T vm = hm ? cu[cix(C, m[0], m[1], m[2])] : (T)0;
        const T vp = hp ? cu[cix(C, p[0], p[1], p[2])] : (T)0;
        if (hm && hp)
            v += del * (T)0.5 * (vp - vm) + (T)0.5 * del * del * (vp - (T)2 * v0 + vm);
        else if (hp)
            v += del * (vp - v0);
        else if (hm)
            v += del * (v0 - vm);
    }
    return v;
}

// Diagonal and off-diagonal parts of (L u)_c = diag u_c - off on level L (coarse level C for
// the coarse-fine ghosts; cu null: zero coarse data).
template <typename T>
AMR_HD inline void cell_op(const Geo& G, const LevT<T>& L, const LevT<T>& C, const int c[3],
                           const T* u, const T* cu, T& diag, T& off) {
    diag = 0;
    off = 0;
    AMR_UNROLL
    for (int d = 0; d < 3; ++d) {   // (static bounds keep the small arrays in registers)
        if (d >= G.dm) break;
        const T ih2 = (T)L.ih2[d];
        AMR_UNROLL
        for (int s = -1; s <= 1; s += 2) {
            const T w = face_b(L, d, c, s) * ih2;
            const int qd = wrap(G, L, d, c[d] + s);
            if (qd < 0) {
                if (s < 0 ? G.dlo[d] : G.dhi[d]) diag += (T)2 * w;
                continue;
            }
            int q[3] = {c[0], c[1], c[2]};
            q[d] = qd;
            const bool qin = inside(L, q);
            const long qc = qin ? cix(L, q[0], q[1], q[2]) : 0;
            if (qin && in_region(L, qc)) {
                diag += w;
                off += w * u[qc];
            } else {
                diag += (T)(2.0 / 3.0) * w;
                if (cu) off += (T)(2.0 / 3.0) * w * coarse_at_ghost(G, C, q, d, cu);
            }
        }
    }
}

// Box coordinates of a cell index.  32-bit unsigned division (several times cheaper than 64-bit
// on the GPU): a level holds at most 2^31 cells, checked where the hierarchy is built, and its
// face arrays fewer than 2^32 entries.
template <typename T>
AMR_HD inline void cell_coords(const LevT<T>& L, long idx, int c[3]) {
    const unsigned u = (unsigned)idx, e0 = (unsigned)L.ext[0], e1 = (unsigned)L.ext[1];
    const unsigned r = u / e0, k = r / e1;
    c[0] = L.lo[0] + (int)(u - r * e0);
    c[1] = L.lo[1] + (int)(r - k * e1);
    c[2] = L.lo[2] + (int)k;
}

// r = f - L u on a region cell, 0 elsewhere.
template <typename T>
AMR_HD inline void defect_cell(const Geo& G, const LevT<T>& L, const LevT<T>& C, long idx,
                               const T* u, const T* cu, const T* f, T* r) {
    if (!in_region(L, idx)) {
        r[idx] = 0;
        return;
    }
    int c[3];
    cell_coords(L, idx, c);
    T dg, off;
    cell_op(G, L, C, c, u, cu, dg, off);
    r[idx] = f[idx] - (dg * u[idx] - off);
}

// Gauss-Seidel update of a region cell of the given colour, zero coarse data.
// Cells of one colour, half a row each: thread t covers row t / hw (hw = ceil(ext0 / 2)) at
// x = 2 (t % hw) + the row's first cell of that colour.  Returns the box index, or -1 past the
// row's end (odd ext0).  t < colour_threads(L) keeps the row inside the box.
template <typename T>
AMR_HD inline long colour_threads(const LevT<T>& L) {
    return (long)((L.ext[0] + 1) / 2) * L.ext[1] * L.ext[2];
}
template <typename T>
AMR_HD inline long colour_cell(const LevT<T>& L, long t, int colour) {
    const unsigned hw = (unsigned)(L.ext[0] + 1) / 2, e1 = (unsigned)L.ext[1];
    const unsigned ut = (unsigned)t, row = ut / hw, kk = row / e1;
    const int j = (int)(row - kk * e1), k = (int)kk;
    const int x0 = (colour + L.lo[0] + L.lo[1] + j + L.lo[2] + k) & 1;
    const int x = 2 * (int)(ut - row * hw) + x0;
    if (x >= L.ext[0]) return -1;
    return (long)x + (long)L.ext[0] * ((long)j + (long)L.ext[1] * k);
}

template <typename T>
AMR_HD inline void gsrb_cell(const Geo& G, const LevT<T>& L, long idx, int colour, T* u,
                             const T* f) {
    int c[3];
    cell_coords(L, idx, c);
    if (((c[0] + c[1] + c[2]) & 1) != colour || !in_region(L, idx)) return;
    T dg, off;
    cell_op<T>(G, L, L, c, u, nullptr, dg, off);
    u[idx] = (f[idx] + off) / dg;
}

// Reflux into a valid coarse cell K (level C) next to cells covered by level F:
// res += (T_coarse - mean T_fine) / h.  uc null: zero coarse data.
template <typename T>
AMR_HD inline void reflux_cell(const Geo& G, const LevT<T>& F, const LevT<T>& C, long kidx,
                               const T* uf, const T* uc, T* res) {
    if (!is_valid(C, kidx)) return;
    int c[3];
    cell_coords(C, kidx, c);
    const int ntan = 1 << (G.dm - 1);
    T acc = 0;
    AMR_UNROLL
    for (int d = 0; d < 3; ++d) {
        if (d >= G.dm) break;
        AMR_UNROLL
        for (int s = -1; s <= 1; s += 2) {
            const int w = wrap(G, C, d, c[d] + s);
            if (w < 0) continue;
            int Q[3] = {c[0], c[1], c[2]};
            Q[d] = w;
            const long qc = cix(C, Q[0], Q[1], Q[2]);
            if (!(C.mask[qc] & kCov)) continue;
            const T Tc = uc ? face_b(C, d, c, s) * (uc[kidx] - uc[qc]) * (T)C.ih[d] : (T)0;
            T Tf = 0;
            AMR_UNROLL
            for (int a = 0; a < 8; ++a) {
                if (a >= (1 << G.dm)) break;
                if ((a >> d) & 1) continue;
                int fc[3] = {0, 0, 0}, gq[3] = {0, 0, 0};
                AMR_UNROLL
                for (int e = 0; e < 3; ++e) {
                    if (e >= G.dm) break;
                    if (e == d) {
                        fc[e] = s > 0 ? 2 * Q[e] : 2 * Q[e] + 1;
                        gq[e] = s > 0 ? 2 * c[e] + 1 : 2 * c[e];
                    } else {
                        fc[e] = gq[e] = 2 * c[e] + ((a >> e) & 1);
                    }
                }
                const T ufv = uf[cix(F, fc[0], fc[1], fc[2])];
                const T g = ufv / (T)3 + (uc ? (T)(2.0 / 3.0) * coarse_at_ghost(G, C, gq, d, uc) : (T)0);
                Tf += face_b(F, d, fc, -s) * (g - ufv) * (T)F.ih[d];
            }
            acc += (Tc - Tf / (T)ntan) * (T)C.ih[d];
        }
    }
    res[kidx] += acc;
}

// Covered coarse cell K (level C) = mean of its children (level F).
template <typename T>
AMR_HD inline void restrict_cell(const Geo& G, const LevT<T>& F, const LevT<T>& C, long kidx,
                                 const T* fine, T* crse) {
    if (!(C.mask[kidx] & kCov)) return;
    int c[3];
    cell_coords(C, kidx, c);
    const int r0 = G.dm > 0 ? 2 : 1, r1 = G.dm > 1 ? 2 : 1, r2 = G.dm > 2 ? 2 : 1;
    T s = 0;
    for (int c2 = 0; c2 < r2; ++c2)
        for (int c1 = 0; c1 < r1; ++c1)
            for (int c0 = 0; c0 < r0; ++c0)
                s += fine[cix(F, c[0] * r0 + c0, c[1] * r1 + c1, c[2] * r2 + c2)];
    crse[kidx] = s / (T)(r0 * r1 * r2);
}

// uf = multilinear interpolation (3/4, 1/4 per direction) of uc on a region cell of level F,
// 0 elsewhere; physical faces reflect (Dirichlet odd, others even).
template <typename T>
AMR_HD inline void prolong_cell(const Geo& G, const LevT<T>& F, const LevT<T>& C, long idx,
                                const T* uc, T* uf) {
    if (!in_region(F, idx)) {
        uf[idx] = 0;
        return;
    }
    int fi[3];
    cell_coords(F, idx, fi);
    int pc[3], off[3];
    for (int d = 0; d < 3; ++d) {
        const bool act = d < G.dm;
        pc[d] = act ? fi[d] >> 1 : fi[d];
        off[d] = act ? ((fi[d] & 1) ? 1 : -1) : 0;
    }
    T s = 0;
    for (int a2 = 0; a2 < (off[2] ? 2 : 1); ++a2)
        for (int a1 = 0; a1 < (off[1] ? 2 : 1); ++a1)
            for (int a0 = 0; a0 < (off[0] ? 2 : 1); ++a0) {
                const int a[3] = {a0, a1, a2};
                T w = 1, sgn = 1;
                int q[3];
                for (int d = 0; d < 3; ++d) {
                    if (!off[d]) {
                        q[d] = pc[d];
                        continue;
                    }
                    w *= a[d] ? (T)0.25 : (T)0.75;
                    const int want = pc[d] + (a[d] ? off[d] : 0);
                    const int got = wrap(G, C, d, want);
                    if (got >= 0) {
                        q[d] = got;
                    } else {
                        q[d] = pc[d];
                        if (want < 0 ? G.dlo[d] : G.dhi[d]) sgn = -sgn;
                    }
                }
                s += w * sgn * uc[cix(C, q[0], q[1], q[2])];
            }
    uf[idx] = s;
}

// Whether the face (d, f) of level L borders a cell of its region.
template <typename T>
AMR_HD inline bool face_in_level(const Geo& G, const LevT<T>& L, int d, const int f[3]) {
    int lo[3] = {f[0], f[1], f[2]}, hi[3] = {f[0], f[1], f[2]};
    lo[d] = wrap(G, L, d, f[d] - 1);
    hi[d] = wrap(G, L, d, f[d]);
    return (lo[d] >= 0 && inside(L, lo) && in_region(L, cix(L, lo[0], lo[1], lo[2]))) ||
           (hi[d] >= 0 && inside(L, hi) && in_region(L, cix(L, hi[0], hi[1], hi[2])));
}

template <typename T>
AMR_HD inline void face_coords(const LevT<T>& L, int d, long idx, int f[3]) {
    const unsigned m0 = (unsigned)(L.ext[0] + (d == 0)), m1 = (unsigned)(L.ext[1] + (d == 1));
    const unsigned u = (unsigned)idx, r = u / m0, k = r / m1;
    f[0] = L.lo[0] + (int)(u - r * m0);
    f[1] = L.lo[1] + (int)(r - k * m1);
    f[2] = L.lo[2] + (int)k;
}

// ml_edge_restriction of one coarse face (direction d): the mean of the fine faces tiling it,
// where the fine level has them.
AMR_HD inline void edge_restrict_face(const Geo& G, const Lev& F, const Lev& C, int d, long idx,
                                      double* uc, const double* uf) {
    int cf[3];
    face_coords(C, d, idx, cf);
    int f0[3];
    for (int e = 0; e < 3; ++e) f0[e] = e < G.dm ? 2 * cf[e] : cf[e];
    if (!face_in_level(G, F, d, f0)) return;
    double s = 0.0;
    int cnt = 0;
    for (int a = 0; a < (1 << G.dm); ++a) {
        if ((a >> d) & 1) continue;
        int f[3] = {f0[0], f0[1], f0[2]};
        for (int e = 0; e < G.dm; ++e)
            if (e != d) f[e] += (a >> e) & 1;
        s += uf[fix(F, d, f[0], f[1], f[2])];
        ++cnt;
    }
    uc[idx] = s / cnt;
}

// Periodic image faces of a fine level's face array gathered from fabs: along a periodic
// direction d spanned by the array box, faces 0 and n are one face stored twice.  A box owns
// face 0 when its cell 0 is in the region, face n when its cell n - 1 is; the caller's fabs set
// only the owned copy, so the other copy is set from it (t: the face's position across d).
AMR_HD inline void sync_periodic_face(const Geo& G, const Lev& L, int d, long t, double* u) {
    if (d >= G.dm || !G.per[d] || L.lo[d] != 0 || L.ext[d] != L.n[d]) return;
    int c[3], e0 = -1, e1 = -1;
    for (int e = 0; e < 3; ++e)
        if (e != d) (e0 < 0 ? e0 : e1) = e;
    c[e0] = L.lo[e0] + (int)(t % L.ext[e0]);
    c[e1] = L.lo[e1] + (int)(t / L.ext[e0]);
    c[d] = 0;
    const bool own0 = in_region(L, cix(L, c[0], c[1], c[2]));
    c[d] = L.n[d] - 1;
    const bool own1 = in_region(L, cix(L, c[0], c[1], c[2]));
    int f[3] = {c[0], c[1], c[2]};
    f[d] = 0;
    const long i0 = fix(L, d, f[0], f[1], f[2]);
    f[d] = L.n[d];
    const long i1 = fix(L, d, f[0], f[1], f[2]);
    if (own0 && !own1) u[i1] = u[i0];
    if (own1 && !own0) u[i0] = u[i1];
}

// Planar beta0 of the face (d, f): beta0_edge along the vertical, beta0 otherwise.
AMR_HD inline double beta0_of_face(const Geo& G, int d, const int f[3], const double* b0,
                                   const double* b0e) {
    const int r = f[G.va];
    return d == G.va ? b0e[r] : b0[r];
}

// rh = -(div(beta0 U) - macrhs) on a region cell (U already holds beta0 U), 0 elsewhere.
AMR_HD inline void divergence_cell(const Geo& G, const Lev& L, long idx, const double* u0,
                                   const double* u1, const double* u2, const double* macrhs,
                                   double* rh) {
    if (!in_region(L, idx)) {
        rh[idx] = 0.0;
        return;
    }
    int c[3];
    cell_coords(L, idx, c);
    const double* u[3] = {u0, u1, u2};
    double dv = 0.0;
    for (int d = 0; d < G.dm; ++d) {
        int hi[3] = {c[0], c[1], c[2]};
        hi[d] += 1;
        dv += (u[d][fix(L, d, hi[0], hi[1], hi[2])] - u[d][fix(L, d, c[0], c[1], c[2])]) / L.h[d];
    }
    if (macrhs) dv -= macrhs[idx];
    rh[idx] = -dv;
}

// Solver coefficient of a face of the level: beta0^p * 2 / (rho_L + rho_R) (mk_mac_coeffs, the
// ghost density the periodic image or the boundary cell); faces off the level are left alone.
AMR_HD inline void coeff_face(const Geo& G, const Lev& L, int d, long idx, const double* rho,
                              const double* b0, const double* b0e, int alt_energy_fix,
                              double* beta) {
    int f[3];
    face_coords(L, d, idx, f);
    if (!face_in_level(G, L, d, f)) return;
    int lo[3] = {f[0], f[1], f[2]}, hi[3] = {f[0], f[1], f[2]};
    const int n = L.n[d];
    lo[d] = f[d] - 1;
    if (lo[d] < 0) lo[d] = G.per[d] ? n - 1 : 0;
    if (hi[d] >= n) hi[d] = G.per[d] ? 0 : n - 1;
    double v = 2.0 / (rho[cix(L, hi[0], hi[1], hi[2])] + rho[cix(L, lo[0], lo[1], lo[2])]);
    if (b0) {
        const double bb = beta0_of_face(G, d, f, b0, b0e);
        v *= bb;
        if (alt_energy_fix) v *= bb;
    }
    beta[idx] = v;
}

// mkumac on a face of the level: beta0 U -= beta_f * G phi; coarse-fine faces use the composite
// ghost (coarse phi cphi of level C), physical faces as on one level.
AMR_HD inline void correct_face(const Geo& G, const Lev& L, const Lev& C, int d, long idx,
                                const double* phi, const double* cphi, const double* beta,
                                double* u) {
    int f[3];
    face_coords(L, d, idx, f);
    if (!face_in_level(G, L, d, f)) return;
    int lo[3] = {f[0], f[1], f[2]}, hi[3] = {f[0], f[1], f[2]};
    lo[d] = wrap(G, L, d, f[d] - 1);
    hi[d] = wrap(G, L, d, f[d]);
    const bool lin = lo[d] >= 0 && inside(L, lo) && in_region(L, cix(L, lo[0], lo[1], lo[2]));
    const bool hin = hi[d] >= 0 && inside(L, hi) && in_region(L, cix(L, hi[0], hi[1], hi[2]));
    const double h = L.h[d];
    double g;
    if (lin && hin) {
        g = (phi[cix(L, hi[0], hi[1], hi[2])] - phi[cix(L, lo[0], lo[1], lo[2])]) / h;
    } else if (hin && lo[d] < 0) {
        g = G.dlo[d] ? 2.0 * phi[cix(L, hi[0], hi[1], hi[2])] / h : 0.0;
    } else if (lin && hi[d] < 0) {
        g = G.dhi[d] ? -2.0 * phi[cix(L, lo[0], lo[1], lo[2])] / h : 0.0;
    } else if (hin) {
        const double pv = phi[cix(L, hi[0], hi[1], hi[2])];
        const double gv = pv / 3.0 + (2.0 / 3.0) * coarse_at_ghost(G, C, lo, d, cphi);
        g = (pv - gv) / h;
    } else {
        const double pv = phi[cix(L, lo[0], lo[1], lo[2])];
        const double gv = pv / 3.0 + (2.0 / 3.0) * coarse_at_ghost(G, C, hi, d, cphi);
        g = (gv - pv) / h;
    }
    u[idx] -= beta[idx] * g;
}

// ---- mixed precision: hand-over between the FP64 solution and the FP32 correction ------------
AMR_HD inline void to_single_cell(long idx, const double* x, float* y) { y[idx] = (float)x[idx]; }
template <typename T>
AMR_HD inline void accumulate_cell(const LevT<T>& L, long idx, double* phi, const float* e) {
    if (in_region(L, idx)) phi[idx] += (double)e[idx];
}

// ---- whole-level-domain arrays <-> box arrays ---------------------------------------------------
template <typename T>
AMR_HD inline long full_cell(const LevT<T>& L, long idx) {
    int c[3];
    cell_coords(L, idx, c);
    return (long)c[0] + (long)L.n[0] * ((long)c[1] + (long)L.n[1] * c[2]);
}
template <typename T>
AMR_HD inline long full_face(const LevT<T>& L, int d, long idx) {
    int f[3];
    face_coords(L, d, idx, f);
    const long m0 = L.n[0] + (d == 0), m1 = L.n[1] + (d == 1);
    return (long)f[0] + m0 * ((long)f[1] + m1 * f[2]);
}

// ---- caller fabs <-> level arrays -------------------------------------------------------------
//
// One fab of the caller's layout on a level: box [lo, hi] in level indices, ng ghost cells,
// natural (Fortran) order over ext[] = box extent + 2 ng (+1 along a face direction); one
// component starting at src (gather) / dst (scatter).
struct FabDesc {
    const double* src;
    double* dst;
    int lo[3], hi[3];
    int ext[3];
    int ng;
    long count;
};

// Level-array index of element e of fab B (dir: face direction, -1 cells).  Returns 1 for the
// box's own cells / faces, 2 for a ghost cell inside the domain (periodic images wrapped), 0 for
// anything else (ghost faces, ghosts beyond a non-periodic domain face).
AMR_HD inline int fab_elem(const Geo& G, const Lev& L, int dir, const FabDesc& B, long e,
                           long* tgt) {
    int a[3];
    a[0] = (int)(e % B.ext[0]);
    const long r = e / B.ext[0];
    a[1] = (int)(r % B.ext[1]);
    a[2] = (int)(r / B.ext[1]);
    int g[3] = {0, 0, 0};
    bool interior = true;
    for (int d = 0; d < G.dm; ++d) {
        g[d] = B.lo[d] - B.ng + a[d];
        const int top = B.hi[d] + (dir == d ? 1 : 0);
        if (g[d] < B.lo[d] || g[d] > top) interior = false;
    }
    if (interior) {
        if (dir < 0 ? !inside(L, g) : !inside_face(L, dir, g)) return 0;
        *tgt = dir < 0 ? cix(L, g[0], g[1], g[2]) : fix(L, dir, g[0], g[1], g[2]);
        return 1;
    }
    if (dir >= 0) return 0;
    for (int d = 0; d < G.dm; ++d) {
        const int q = wrap(G, L, d, g[d]);
        if (q < 0) return 0;
        g[d] = q;
    }
    if (!inside(L, g)) return 0;
    *tgt = cix(L, g[0], g[1], g[2]);
    return 2;
}

// Gather element e of fab B into the level array: the box's own entries always, ghost cells
// (with_ghosts) only where the cell lies outside the level's region.
AMR_HD inline void fab_gather_elem(const Geo& G, const Lev& L, int dir, const FabDesc& B, long e,
                                   int with_ghosts, double* level) {
    long t;
    const int kind = fab_elem(G, L, dir, B, e, &t);
    if (kind == 1 || (kind == 2 && with_ghosts && !in_region(L, t))) level[t] = B.src[e];
}

// Scatter the box's own entries of the level array into element e of fab B.
AMR_HD inline void fab_scatter_elem(const Geo& G, const Lev& L, int dir, const FabDesc& B, long e,
                                    const double* level) {
    long t;
    if (fab_elem(G, L, dir, B, e, &t) == 1) B.dst[e] = level[t];
}

// create_umac_grown (Source/macproject.f90:264-272; the routine is FBoxLib's and not in the
// MAESTRO tree, so it is written here from what it is for): after the projection a fine level's
// edge velocities in the ghost faces of its fabs come from the level itself where the face
// borders one of the level's cells (a neighbouring box's face, periodic images wrapped: the
// fill_boundary the routine ends with), else from the coarser level -- piecewise constant
// across the face, linear along its normal: a fine face on a coarse face plane takes that
// coarse face's value, one between two coarse planes their mean.  g: the ghost face (index
// along dir, cells along the other directions) in the fine level's domain.  Returns false for
// a face beyond a non-periodic domain face (the caller's physical-boundary fill) and leaves
// *out alone.
AMR_HD inline bool grow_face(const Geo& G, const Lev& F, const Lev& C, int dir, const int g_in[3],
                             const double* uf, const double* uc, double* out) {
    int g[3] = {g_in[0], g_in[1], g_in[2]};
    for (int d = 0; d < G.dm; ++d) {
        const int n = F.n[d];
        if (d == dir) {   // faces 0 .. n
            if (g[d] < 0 || g[d] > n) {
                if (!G.per[d]) return false;
                g[d] += g[d] < 0 ? n : -n;
            }
        } else {
            const int q = wrap(G, F, d, g[d]);
            if (q < 0) return false;
            g[d] = q;
        }
    }
    // the two cells the face separates, when they exist
    const int n = F.n[dir];
    bool own = false;
    for (int s = 0; s < 2 && !own; ++s) {
        int cc[3] = {g[0], g[1], g[2]};
        cc[dir] = g[dir] - 1 + s;
        if (cc[dir] < 0 || cc[dir] >= n) {
            if (!G.per[dir]) continue;
            cc[dir] += cc[dir] < 0 ? n : -n;
        }
        own = inside(F, cc) && (F.mask[cix(F, cc[0], cc[1], cc[2])] & kIn);
    }
    if (own) {
        if (!inside_face(F, dir, g)) return false;
        *out = uf[fix(F, dir, g[0], g[1], g[2])];
        return true;
    }
    int c[3] = {g[0] >> 1, g[1] >> 1, g[2] >> 1};
    if ((g[dir] & 1) == 0) {
        c[dir] = g[dir] >> 1;
        if (!inside_face(C, dir, c)) return false;
        *out = uc[fix(C, dir, c[0], c[1], c[2])];
        return true;
    }
    int c1[3] = {c[0], c[1], c[2]};
    c[dir] = (g[dir] - 1) >> 1;
    c1[dir] = (g[dir] + 1) >> 1;
    if (!inside_face(C, dir, c) || !inside_face(C, dir, c1)) return false;
    *out = 0.5 * (uc[fix(C, dir, c[0], c[1], c[2])] + uc[fix(C, dir, c1[0], c1[1], c1[2])]);
    return true;
}

// The ghost faces of element e of face fab B (dir) by grow_face; the box's own faces and faces
// beyond a non-periodic domain face are left alone.
AMR_HD inline void fab_grow_elem(const Geo& G, const Lev& F, const Lev& C, int dir,
                                 const FabDesc& B, long e, const double* uf, const double* uc) {
    int a[3];
    a[0] = (int)(e % B.ext[0]);
    const long r = e / B.ext[0];
    a[1] = (int)(r % B.ext[1]);
    a[2] = (int)(r / B.ext[1]);
    int g[3] = {0, 0, 0};
    bool interior = true;
    for (int d = 0; d < G.dm; ++d) {
        g[d] = B.lo[d] - B.ng + a[d];
        const int top = B.hi[d] + (dir == d ? 1 : 0);
        if (g[d] < B.lo[d] || g[d] > top) interior = false;
    }
    if (interior) return;
    double v;
    if (grow_face(G, F, C, dir, g, uf, uc, &v)) B.dst[e] = v;
}

// ---- the multi-level cycle and the projection steps -------------------------------------------
//
// E provides, for levels l = 0 .. nlev-1 (arrays are E's own memory):
//   int nlev; Geo geo; bool singular; Lev lev(l);
//   double* buf(l, which)          work arrays: kF, kPhi, kRes, kUu, kHold, kTmp, kDu, kRh
//   double* beta(l, d)             face coefficients of level l
//   void defect(l, u, cu, f, r)    r = f - L u (cu: level l-1 data for the C-F ghosts or null)
//   void gsrb(l, u, f, nu)         nu red/black sweeps, zero coarse data
//   void reflux(l, uf, uc, res)    into level l-1 from level l
//   void restrict_cov(l, fine, crse)
//   void prolong(l, uc, uf)        level l-1 -> level l
//   void axpy3(l, uu, hold, du)    uu += hold + du on the region
//   void add_region(l, phi, uu)    phi += uu on the region
//   void zero(l, x)
//   double valid_max(which)        max over the valid cells of all levels (host value)
//   double valid_mean(which)       volume-weighted mean over the valid cells (host value)
//   void sub_valid(which, m)       x -= m on the valid cells of all levels
//   int level0_correction(rhs, e)  one V-cycle of the level-0 multigrid, zero guess, constant
//                                  removed when singular; returns 0 or an error code
//   int error()                    sticky launch / device error (0: none)
// and for the projection:
//   void scale_b0(l, mult)  edge_restrict(l)  divergence(l)  coeffs(l)  correct(l)
enum { kF = 0, kPhi, kRes, kUu, kHold, kTmp, kDu, kRh, kNumBufs };

struct SolveStats {
    int status;      // 0 converged, 1 not converged, < 0 error
    int cycles;
    double fnorm;
    double resid0;
    double rel_resid;
    int nhist;
    double hist[64];
};

// Composite defect of buf(kPhi) against buf(kF) into buf(kRes) on every level.
template <class E>
void composite_defect(E& ex) {
    const int nl = ex.nlev;
    for (int l = 0; l < nl; ++l)
        ex.defect(l, ex.buf(l, kPhi), l ? ex.buf(l - 1, kPhi) : nullptr, ex.buf(l, kF),
                  ex.buf(l, kRes));
    for (int l = nl - 1; l >= 1; --l) {
        ex.reflux(l, ex.buf(l, kPhi), ex.buf(l - 1, kPhi), ex.buf(l - 1, kRes));
        ex.restrict_cov(l, ex.buf(l, kRes), ex.buf(l - 1, kRes));
    }
}

template <class E>
double composite_residual(E& ex) {
    composite_defect(ex);
    return ex.valid_max(kRes);
}

template <class E>
int ml_vcycle(E& ex, int nu1, int nu2) {
    const int nl = ex.nlev;
    for (int l = nl - 1; l >= 1; --l) {
        ex.zero(l, ex.buf(l, kUu));
        ex.gsrb(l, ex.buf(l, kUu), ex.buf(l, kRes), nu1);
        ex.defect(l, ex.buf(l, kUu), nullptr, ex.buf(l, kRes), ex.buf(l, kTmp));
        ex.swap_bufs(l, kRes, kTmp);
        ex.copy(l, ex.buf(l, kHold), ex.buf(l, kUu));
        ex.restrict_cov(l, ex.buf(l, kRes), ex.buf(l - 1, kRes));
        ex.reflux(l, ex.buf(l, kUu), nullptr, ex.buf(l - 1, kRes));
    }
    int rc = ex.level0_correction(ex.buf(0, kRes), ex.buf(0, kUu));
    if (rc) return rc;
    for (int l = 1; l < nl; ++l) {
        ex.prolong(l, ex.buf(l - 1, kUu), ex.buf(l, kUu));
        ex.defect(l, ex.buf(l, kUu), ex.buf(l - 1, kUu), ex.buf(l, kRes), ex.buf(l, kTmp));
        ex.zero(l, ex.buf(l, kDu));
        ex.gsrb(l, ex.buf(l, kDu), ex.buf(l, kTmp), nu2);
        ex.axpy3(l, ex.buf(l, kUu), ex.buf(l, kHold), ex.buf(l, kDu));
    }
    for (int l = 0; l < nl; ++l) ex.add_region(l, ex.buf(l, kPhi), ex.buf(l, kUu));
    for (int l = nl - 1; l >= 1; --l) ex.restrict_cov(l, ex.buf(l, kPhi), ex.buf(l - 1, kPhi));
    return ex.error();
}

// Composite solve of L phi = f with f in buf(l, kF) and the initial guess in buf(l, kPhi) (only
// region cells are read).  rel_eps / abs_eps (<= 0: unused) as in mac_opts.
template <class E>
int amr_solve(E& ex, double rel_eps, double abs_eps, int max_cycles, int nu1, int nu2,
              SolveStats* S) {
    const int nl = ex.nlev;
    *S = SolveStats{};
    if (ex.singular) ex.sub_valid(kF, ex.valid_mean(kF));
    for (int l = nl - 1; l >= 1; --l) ex.restrict_cov(l, ex.buf(l, kPhi), ex.buf(l - 1, kPhi));
    const double fnorm = ex.valid_max(kF);
    S->fnorm = fnorm;
    if (!(fnorm > 0.0)) {
        for (int l = 0; l < nl; ++l) ex.zero(l, ex.buf(l, kPhi));
        S->status = std::isnan(fnorm) ? -1 : 0;
        return ex.error() ? ex.error() : S->status;
    }
    auto converged = [&](double r) {
        return r <= rel_eps * fnorm || (abs_eps > 0.0 && r <= abs_eps);
    };
    double res = composite_residual(ex);
    S->resid0 = res;
    int it = 0;
    while (!converged(res) && it < max_cycles && !std::isnan(res)) {
        int rc = ml_vcycle(ex, nu1, nu2);
        if (rc) {
            S->status = rc;
            return rc;
        }
        ++it;
        res = composite_residual(ex);
        if (S->nhist < 64) S->hist[S->nhist++] = res / fnorm;
    }
    S->cycles = it;
    S->rel_resid = res / fnorm;
    S->status = converged(res) ? 0 : 1;
    return ex.error() ? ex.error() : S->status;
}

// Mixed precision: the FP64 composite residual, `inner` FP32 multi-level V-cycles on it from a
// zero correction (ex32: FP32 copies of the levels and coefficients; its level-0 correction is
// the FP64 one-level V-cycle), the correction added to the FP64 solution, until the FP64
// composite residual meets the tolerance.
template <class E, class E32>
int amr_solve_mixed(E& ex, E32& ex32, double rel_eps, double abs_eps, int max_iters, int nu1,
                    int nu2, int inner, SolveStats* S) {
    const int nl = ex.nlev;
    *S = SolveStats{};
    if (ex.singular) ex.sub_valid(kF, ex.valid_mean(kF));
    for (int l = nl - 1; l >= 1; --l) ex.restrict_cov(l, ex.buf(l, kPhi), ex.buf(l - 1, kPhi));
    const double fnorm = ex.valid_max(kF);
    S->fnorm = fnorm;
    if (!(fnorm > 0.0)) {
        for (int l = 0; l < nl; ++l) ex.zero(l, ex.buf(l, kPhi));
        S->status = std::isnan(fnorm) ? -1 : 0;
        return ex.error() ? ex.error() : S->status;
    }
    auto converged = [&](double r) {
        return r <= rel_eps * fnorm || (abs_eps > 0.0 && r <= abs_eps);
    };
    double res = composite_residual(ex);
    S->resid0 = res;
    int it = 0;
    while (!converged(res) && it < max_iters && !std::isnan(res)) {
        for (int l = 0; l < nl; ++l) {
            ex.to_single(l, ex.buf(l, kRes), ex32.buf(l, kF));
            ex32.zero(l, ex32.buf(l, kPhi));
        }
        for (int v = 0; v < inner; ++v) {
            if (v == 0)
                for (int l = 0; l < nl; ++l) ex32.copy(l, ex32.buf(l, kRes), ex32.buf(l, kF));
            else
                composite_defect(ex32);
            int rc = ml_vcycle(ex32, nu1, nu2);
            if (rc) {
                S->status = rc;
                return rc;
            }
        }
        for (int l = 0; l < nl; ++l) ex.accumulate(l, ex.buf(l, kPhi), ex32.buf(l, kPhi));
        for (int l = nl - 1; l >= 1; --l) ex.restrict_cov(l, ex.buf(l, kPhi), ex.buf(l - 1, kPhi));
        res = composite_residual(ex);
        ++it;
        if (S->nhist < 64) S->hist[S->nhist++] = res / fnorm;
        if (ex.error() || ex32.error()) return ex.error() ? ex.error() : ex32.error();
    }
    S->cycles = it * inner;
    S->rel_resid = res / fnorm;
    S->status = converged(res) ? 0 : 1;
    return ex.error() ? ex.error() : S->status;
}

// Multi-level MAC projection (Source/macproject.f90:51-328, nlevs > 1) on the executor's level
// arrays: velocities, density, macrhs and beta0 already loaded; phi in buf(l, kPhi).
template <class E, class E32 = E>
int amr_project(E& ex, double rel_eps, double abs_eps, int max_cycles, int nu1, int nu2,
                SolveStats* S, E32* ex32 = nullptr, int inner = 0) {
    const int nl = ex.nlev;
    for (int l = 0; l < nl; ++l) ex.scale_b0(l, true);
    for (int l = nl - 1; l >= 1; --l) ex.edge_restrict(l);
    for (int l = 0; l < nl; ++l) ex.divergence(l);          // buf(l, kRh)
    for (int l = nl - 1; l >= 1; --l) ex.restrict_cov(l, ex.buf(l, kRh), ex.buf(l - 1, kRh));
    for (int l = 0; l < nl; ++l) {
        ex.coeffs(l);
        ex.copy(l, ex.buf(l, kF), ex.buf(l, kRh));
    }
    int rc = ex.prepare_level0();
    if (rc) return rc;
    if constexpr (!std::is_same<E32, E>::value) {
        if (ex32) {
            ex.faces_to_single();   // FP32 face coefficients of every level
            rc = amr_solve_mixed(ex, *ex32, rel_eps, abs_eps, max_cycles, nu1, nu2, inner, S);
        } else {
            rc = amr_solve(ex, rel_eps, abs_eps, max_cycles, nu1, nu2, S);
        }
    } else {
        rc = amr_solve(ex, rel_eps, abs_eps, max_cycles, nu1, nu2, S);
    }
    if (rc < 0) return rc;
    const int status = rc;
    for (int l = 0; l < nl; ++l) ex.correct(l);
    for (int l = nl - 1; l >= 1; --l) ex.edge_restrict(l);
    for (int l = 0; l < nl; ++l) ex.scale_b0(l, false);
    for (int l = nl - 1; l >= 1; --l) ex.edge_restrict(l);
    rc = ex.error();
    return rc ? rc : status;
}

}  // namespace amr
}  // namespace mac
