// Nodal (HG) projection on one level: the node- and cell-wise arithmetic, and the nodal V-cycle
// and projection steps written once against an executor.
//
// MAESTRO's hgproject (Source/hgproject.f90:32-264) projects the cell-centred velocity with a
// node-centred potential: hg_multigrid (Source/hg_multigrid.f90:18-239) forms the coefficient
// sigma = beta0 / rhohalf per cell (0 outside non-periodic faces), the node-centred divergence
// of beta0 U and solves L phi = DU - nodalrhs with FBoxLib's nodal multigrid; mkgphi takes the
// cell gradient of phi and hg_update corrects U, pi and gpi per projection type.
//
// Storage: natural layout, FP64.  Cells n[d] per active direction; nodes n[d] + 1 per active
// direction, the node n[d] of a periodic direction being the image of node 0 (kernels always
// read through node_wrap, images are refreshed only for the caller's output).  Nodes on an
// outflow (Dirichlet) face hold 0.  Vector cell fields are component-major (d * ncell + c).
//
// Operators (the discretisation of Docs/mg/mg.tex:479-500):
//   dense : (L phi)_p = - sum_{cells c of p} sigma_c sum_{nodes m of c} sum_d h_d^-2
//           S(p_d, m_d) prod_{e != d} M(p_e, m_e) phi_m   -- the (bi/tri)linear finite-element
//           stiffness over the nodal volume, S = [[1,-1],[-1,1]], M = [[1/3,1/6],[1/6,1/3]];
//   cross : (L phi)_p = sum_d h_d^-2 sum_s sigma_edge (phi_{p+s e_d} - phi_p), sigma_edge the
//           mean of sigma over the 2^(dm-1) cells along the edge;
//   DU_p  = sum_d h_d^-1 2^(1-dm) [sum u_d over the cells on the + side of p - the same on the
//           - side] (U = 0 outside non-periodic faces);
//   gphi  = the cell gradient: mean of the nodal differences across the cell (mkgphi).
// Multigrid: 2^dm-colour Gauss-Seidel (node parity), full-weighting restriction of the defect,
// multilinear prolongation, coarse sigma = mean of the fine cells, Gauss-Seidel sweeps on the
// coarsest level.
#pragma once

#include <cmath>
#include <cstdint>
#include <type_traits>
#include <utility>

#if defined(__CUDACC__)
#define HG_HD __host__ __device__
#else
#define HG_HD
#endif
#if defined(__CUDA_ARCH__)
#define HG_UNROLL _Pragma("unroll")
#else
#define HG_UNROLL
#endif

namespace mac {
namespace hg {

constexpr int kMaxLevels = 24;
enum { kInitial = 1, kDivuIters = 2, kPressureIters = 3, kRegular = 4 };

struct Geo {
    int dm;
    int per[3];
    int dlo[3], dhi[3];
    int dense;
};

// Inflow faces of the divergence: face f = 2 d + side (side 0 low, 1 high) is an inflow face when
// off[f] >= 0; w + off[f] then holds the wall value of beta0 U_d there for each cell of the face,
// the face's other directions in Fortran order (the cells a ghost layer outside it would hold).
struct Wall {
    const double* w;
    long off[6];
};

// A level in the precision T of its coefficients and smoother (FP64; FP32 for the inner cycles
// of the mixed-precision solve).
template <typename T>
struct LevT {
    int n[3];          // cells (1 along inactive directions)
    int nn[3];         // node storage (n + 1 along active directions)
    double h[3];
    double ih[3];      // 1 / h (set by set_dense_weights: the one-pass cell and node functions
                       // multiply, FP64 division being slow on the GPU)
    const T* sig;      // cell coefficients
    // dense stencil: finite-element weight of a cell between its corners a and b, which depends
    // on a ^ b only (set by set_dense_weights)
    T kw[8];
};
using Lev = LevT<double>;

// kw[x] = sum_d h_d^-2 S(x_d) prod_{e != d} M(x_e) with S(0) = 1, S(1) = -1, M(0) = 1/3,
// M(1) = 1/6 (x_d = 1: the two corners differ along d).
template <typename T>
HG_HD inline void set_dense_weights(int dm, LevT<T>& L) {
    for (int d = 0; d < 3; ++d) L.ih[d] = 1.0 / L.h[d];
    for (int x = 0; x < 8; ++x) {
        double k = 0.0;
        for (int d = 0; d < dm; ++d) {
            double t = (((x >> d) & 1) ? -1.0 : 1.0) / (L.h[d] * L.h[d]);
            for (int e = 0; e < dm; ++e)
                if (e != d) t *= ((x >> e) & 1) ? 1.0 / 6.0 : 1.0 / 3.0;
            k += t;
        }
        L.kw[x] = (T)(x < (1 << dm) ? k : 0.0);
    }
}

template <typename T>
HG_HD inline long nix(const LevT<T>& L, int i, int j, int k) {
    return (long)i + (long)L.nn[0] * ((long)j + (long)L.nn[1] * k);
}
template <typename T>
HG_HD inline long cix(const LevT<T>& L, int i, int j, int k) {
    return (long)i + (long)L.n[0] * ((long)j + (long)L.n[1] * k);
}
template <typename T>
HG_HD inline long nnodes(const LevT<T>& L) { return (long)L.nn[0] * L.nn[1] * L.nn[2]; }
template <typename T>
HG_HD inline long ncells(const LevT<T>& L) { return (long)L.n[0] * L.n[1] * L.n[2]; }

// Coordinates of a node / cell index (32-bit: a level holds fewer than 2^31 nodes, checked where
// the hierarchy is built; 32-bit division is several times cheaper than 64-bit on the GPU).
template <typename T>
HG_HD inline void node_coords(const LevT<T>& L, long idx, int p[3]) {
    const unsigned u = (unsigned)idx, n0 = (unsigned)L.nn[0], n1 = (unsigned)L.nn[1];
    const unsigned r = u / n0;
    p[0] = (int)(u - r * n0);
    p[2] = (int)(r / n1);
    p[1] = (int)(r - (unsigned)p[2] * n1);
}
template <typename T>
HG_HD inline void cell_coords(const LevT<T>& L, long idx, int c[3]) {
    const unsigned u = (unsigned)idx, n0 = (unsigned)L.n[0], n1 = (unsigned)L.n[1];
    const unsigned r = u / n0;
    c[0] = (int)(u - r * n0);
    c[2] = (int)(r / n1);
    c[1] = (int)(r - (unsigned)c[2] * n1);
}

// Periodic fold of q onto [0, n): every caller passes a q within a few periods of the range
// (a node or cell index +- 1, or 2 P + a of the restriction), so a few adds replace the modulo.
HG_HD inline int fold_periodic(int q, int n) {
    while (q < 0) q += n;
    while (q >= n) q -= n;
    return q;
}
// Node index q along d folded onto the carrying node (periodic wrap); -1 outside.
template <typename T>
HG_HD inline int node_wrap(const Geo& G, const LevT<T>& L, int d, int q) {
    if (d >= G.dm) return q == 0 ? 0 : -1;
    const int n = L.n[d];
    if (G.per[d]) return fold_periodic(q, n);
    return (q < 0 || q > n) ? -1 : q;
}
template <typename T>
HG_HD inline int cell_wrap(const Geo& G, const LevT<T>& L, int d, int c) {
    if (d >= G.dm) return c == 0 ? 0 : -1;
    const int n = L.n[d];
    if (G.per[d]) return fold_periodic(c, n);
    return (c < 0 || c >= n) ? -1 : c;
}
// An unknown: not a periodic image, not on an outflow face.
template <typename T>
HG_HD inline bool is_unknown(const Geo& G, const LevT<T>& L, const int p[3]) {
    HG_UNROLL
    for (int d = 0; d < 3; ++d) {   // (a static bound keeps p[] in registers)
        if (d >= G.dm) break;
        if (G.per[d]) {
            if (p[d] == L.n[d]) return false;
        } else if ((p[d] == 0 && G.dlo[d]) || (p[d] == L.n[d] && G.dhi[d])) {
            return false;
        }
    }
    return true;
}

// (L phi)_p = diag * phi_p - off; DM = G.dm as a compile-time constant, so the corner loops
// unroll and the weight table is indexed statically.
template <int DM, typename T>
HG_HD inline void node_op_dm(const Geo& G, const LevT<T>& L, const int p[3], const T* phi,
                             T& diag, T& off) {
    constexpr int dm = DM;
    T dK = 0, oK = 0;
    if (G.dense) {
        const long pi = nix(L, p[0], p[1], p[2]);
        HG_UNROLL
        for (int a = 0; a < (1 << dm); ++a) {   // a: the corner of cell c that p is
            int c[3] = {0, 0, 0};
            bool out = false;
            HG_UNROLL
            for (int d = 0; d < dm; ++d) {
                const int cw = cell_wrap(G, L, d, p[d] - ((a >> d) & 1));
                if (cw < 0) out = true;
                c[d] = cw;
            }
            if (out) continue;
            const T s = L.sig[cix(L, c[0], c[1], c[2])];
            T acc = 0;
            HG_UNROLL
            for (int b = 0; b < (1 << dm); ++b) {
                if (b == a) continue;
                int m[3] = {0, 0, 0};
                HG_UNROLL
                for (int d = 0; d < dm; ++d) m[d] = node_wrap(G, L, d, c[d] + ((b >> d) & 1));
                const long mi = nix(L, m[0], m[1], m[2]);
                if (mi == pi)   // a periodic wrap of extent 1 folds a corner onto p
                    dK += s * L.kw[a ^ b];
                else
                    acc += L.kw[a ^ b] * phi[mi];
            }
            dK += s * L.kw[0];
            oK -= s * acc;
        }
        diag = -dK;
        off = -oK;
    } else {
        HG_UNROLL
        for (int d = 0; d < dm; ++d)
            HG_UNROLL
            for (int sd = -1; sd <= 1; sd += 2) {
                const int q = node_wrap(G, L, d, p[d] + sd);
                if (q < 0) continue;
                T sum = 0;
                int cnt = 0;
                HG_UNROLL
                for (int a = 0; a < (1 << dm); ++a) {
                    if ((a >> d) & 1) continue;
                    int c[3] = {0, 0, 0};
                    bool out = false;
                    HG_UNROLL
                    for (int e = 0; e < dm; ++e) {
                        const int want = e == d ? (sd < 0 ? p[d] - 1 : p[d]) : p[e] - ((a >> e) & 1);
                        const int cw = cell_wrap(G, L, e, want);
                        if (cw < 0) out = true;
                        c[e] = cw;
                    }
                    ++cnt;
                    if (!out) sum += L.sig[cix(L, c[0], c[1], c[2])];
                }
                const T se = sum / (T)cnt / (T)(L.h[d] * L.h[d]);
                int qq[3] = {p[0], p[1], p[2]};
                qq[d] = q;
                dK -= se;
                oK -= se * phi[nix(L, qq[0], qq[1], qq[2])];
            }
        diag = dK;
        off = oK;
    }
}

template <typename T>
HG_HD inline void node_op(const Geo& G, const LevT<T>& L, const int p[3], const T* phi, T& diag,
                          T& off) {
    if (G.dm == 3)
        node_op_dm<3>(G, L, p, phi, diag, off);
    else
        node_op_dm<2>(G, L, p, phi, diag, off);
}

// Row p of the operator as weights on nodes: add(m, w) for every term w * phi_m of (L phi)_p,
// with m the node storage index after the periodic fold (the diagonal term has m = the index of
// p); the same terms node_op sums, so sum_m w_m phi_m = diag * phi_p - off.
template <typename T, class Add>
HG_HD inline void node_row(const Geo& G, const LevT<T>& L, const int p[3], Add add) {
    const int dm = G.dm;
    const long pi = nix(L, p[0], p[1], p[2]);
    if (G.dense) {
        for (int a = 0; a < (1 << dm); ++a) {
            int c[3] = {0, 0, 0};
            bool out = false;
            for (int d = 0; d < dm; ++d) {
                const int cw = cell_wrap(G, L, d, p[d] - ((a >> d) & 1));
                if (cw < 0) out = true;
                c[d] = cw;
            }
            if (out) continue;
            const T s = L.sig[cix(L, c[0], c[1], c[2])];
            for (int b = 0; b < (1 << dm); ++b) {
                if (b == a) continue;
                int m[3] = {0, 0, 0};
                for (int d = 0; d < dm; ++d) m[d] = node_wrap(G, L, d, c[d] + ((b >> d) & 1));
                add(nix(L, m[0], m[1], m[2]), -(s * L.kw[a ^ b]));
            }
            add(pi, -(s * L.kw[0]));
        }
    } else {
        for (int d = 0; d < dm; ++d)
            for (int sd = -1; sd <= 1; sd += 2) {
                const int q = node_wrap(G, L, d, p[d] + sd);
                if (q < 0) continue;
                T sum = 0;
                int cnt = 0;
                for (int a = 0; a < (1 << dm); ++a) {
                    if ((a >> d) & 1) continue;
                    int c[3] = {0, 0, 0};
                    bool out = false;
                    for (int e = 0; e < dm; ++e) {
                        const int want = e == d ? (sd < 0 ? p[d] - 1 : p[d]) : p[e] - ((a >> e) & 1);
                        const int cw = cell_wrap(G, L, e, want);
                        if (cw < 0) out = true;
                        c[e] = cw;
                    }
                    ++cnt;
                    if (!out) sum += L.sig[cix(L, c[0], c[1], c[2])];
                }
                const T se = sum / (T)cnt / (T)(L.h[d] * L.h[d]);
                int qq[3] = {p[0], p[1], p[2]};
                qq[d] = q;
                add(pi, -se);
                add(nix(L, qq[0], qq[1], qq[2]), se);
            }
    }
}

// r = f - L phi on the unknowns, 0 elsewhere.
template <typename T>
HG_HD inline void defect_node(const Geo& G, const LevT<T>& L, long idx, const T* phi, const T* f,
                              T* r) {
    int p[3];
    node_coords(L, idx, p);
    if (!is_unknown(G, L, p)) {
        r[idx] = 0;
        return;
    }
    T dg, off;
    node_op(G, L, p, phi, dg, off);
    r[idx] = f[idx] - (dg * phi[idx] - off);
}

// Nodes of one colour (parity pattern `colour` of the node coordinates): how many, and the k-th.
template <typename T>
HG_HD inline long colour_count(const Geo& G, const LevT<T>& L, int colour) {
    long m = 1;
    for (int d = 0; d < G.dm; ++d) m *= (L.nn[d] - ((colour >> d) & 1) + 1) / 2;
    return m;
}
template <typename T>
HG_HD inline void colour_node(const Geo& G, const LevT<T>& L, int colour, long k, int p[3]) {
    p[0] = p[1] = p[2] = 0;
    unsigned u = (unsigned)k;
    HG_UNROLL
    for (int d = 0; d < 3; ++d) {   // (a static bound keeps p[] in registers)
        if (d >= G.dm) break;
        const int b = (colour >> d) & 1;
        const unsigned m = (unsigned)((L.nn[d] - b + 1) / 2);
        const unsigned qd = u / m;
        p[d] = 2 * (int)(u - qd * m) + b;
        u = qd;
    }
}

// Gauss-Seidel update of the k-th node of a colour (nodes of one colour share no cell, so a
// colour updates in parallel).
template <typename T>
HG_HD inline void gs_node(const Geo& G, const LevT<T>& L, long k, int colour, T* phi, const T* f) {
    int p[3];
    colour_node(G, L, colour, k, p);
    if (!is_unknown(G, L, p)) return;
    const long idx = nix(L, p[0], p[1], p[2]);
    T dg, off;
    node_op(G, L, p, phi, dg, off);
    phi[idx] = (f[idx] + off) / dg;
}

// Coarse right-hand side = full-weighting restriction of the fine defect (coarse node P <- fine
// nodes 2P + a, a in {-1,0,1}^dm, weights prod (1 or 1/2), divided by 2^dm).
template <typename T>
HG_HD inline void restrict_node(const Geo& G, const LevT<T>& F, const LevT<T>& K, long idx,
                                const T* rF, T* fK) {
    int P[3];
    node_coords(K, idx, P);
    if (!is_unknown(G, K, P)) {
        fK[idx] = 0;
        return;
    }
    const int dm = G.dm;
    T s = 0;
    // a coarse node whose fine neighbours 2P-1 .. 2P+1 need no fold: direct offsets, the same
    // terms in the same order as below
    bool inner = true;
    HG_UNROLL
    for (int d = 0; d < 3; ++d) {
        if (d >= dm) break;
        inner = inner && P[d] >= 1 && 2 * P[d] + 1 <= F.n[d] - 1;
    }
    if (inner) {
        const long st1 = F.nn[0], st2 = (long)F.nn[0] * F.nn[1];
        const T* r = rF + nix(F, 2 * P[0], dm > 1 ? 2 * P[1] : 0, dm > 2 ? 2 * P[2] : 0);
        HG_UNROLL
        for (int a2 = -1; a2 <= 1; ++a2)
            HG_UNROLL
            for (int a1 = -1; a1 <= 1; ++a1)
                HG_UNROLL
                for (int a0 = -1; a0 <= 1; ++a0) {
                    if ((dm < 3 && a2 != 0) || (dm < 2 && a1 != 0)) continue;
                    T w = 1;
                    if (a0) w *= (T)0.5;
                    if (a1) w *= (T)0.5;
                    if (a2) w *= (T)0.5;
                    s += w * r[a0 + a1 * st1 + a2 * st2];
                }
        fK[idx] = s * (dm == 3 ? (T)0.125 : (dm == 2 ? (T)0.25 : (T)0.5));   // 2^-dm, exact
        return;
    }
    // (static bounds, the same terms in the same order: the small arrays stay in registers)
    HG_UNROLL
    for (int a2 = -1; a2 <= 1; ++a2)
        HG_UNROLL
        for (int a1 = -1; a1 <= 1; ++a1)
            HG_UNROLL
            for (int a0 = -1; a0 <= 1; ++a0) {
                if ((dm < 3 && a2 != 0) || (dm < 2 && a1 != 0)) continue;
                const int a[3] = {a0, a1, a2};
                int q[3] = {0, 0, 0};
                T w = 1;
                bool out = false;
                HG_UNROLL
                for (int d = 0; d < 3; ++d) {
                    if (d >= dm) break;
                    if (a[d]) w *= (T)0.5;
                    const int qq = node_wrap(G, F, d, 2 * P[d] + a[d]);
                    if (qq < 0) out = true;
                    q[d] = qq;
                }
                if (!out) s += w * rF[nix(F, q[0], q[1], q[2])];
            }
    fK[idx] = s * (dm == 3 ? (T)0.125 : (dm == 2 ? (T)0.25 : (T)0.5));   // 2^-dm, exact
}

// Fine unknowns += multilinear interpolation of the coarse correction.
template <typename T>
HG_HD inline void prolong_node(const Geo& G, const LevT<T>& K, const LevT<T>& F, long idx,
                               const T* eK, T* phiF) {
    int p[3];
    node_coords(F, idx, p);
    if (!is_unknown(G, F, p)) return;
    const int dm = G.dm;
    int lo[3] = {0, 0, 0}, odd[3] = {0, 0, 0};
    HG_UNROLL
    for (int d = 0; d < 3; ++d) {   // (static bounds keep the small arrays in registers)
        if (d >= dm) break;
        lo[d] = p[d] >> 1;
        odd[d] = p[d] & 1;
    }
    T s = 0;
    // a fine node whose coarse parents need no fold: direct offsets, the same terms in the same
    // order as below
    bool inner = true;
    HG_UNROLL
    for (int d = 0; d < 3; ++d) {
        if (d >= dm) break;
        inner = inner && p[d] <= F.n[d] - 2;
    }
    if (inner) {
        const long st1 = K.nn[0], st2 = (long)K.nn[0] * K.nn[1];
        const T* e = eK + nix(K, lo[0], lo[1], lo[2]);
        T w = 1;
        HG_UNROLL
        for (int d = 0; d < 3; ++d) {
            if (d >= dm) break;
            if (odd[d]) w *= (T)0.5;
        }
        HG_UNROLL
        for (int a2 = 0; a2 <= 1; ++a2)
            HG_UNROLL
            for (int a1 = 0; a1 <= 1; ++a1)
                HG_UNROLL
                for (int a0 = 0; a0 <= 1; ++a0) {
                    if (a2 > odd[2] || a1 > odd[1] || a0 > odd[0]) continue;
                    s += w * e[a0 + a1 * st1 + a2 * st2];
                }
        phiF[idx] += s;
        return;
    }
    HG_UNROLL
    for (int a2 = 0; a2 <= 1; ++a2)
        HG_UNROLL
        for (int a1 = 0; a1 <= 1; ++a1)
            HG_UNROLL
            for (int a0 = 0; a0 <= 1; ++a0) {
                if (a2 > odd[2] || a1 > odd[1] || a0 > odd[0]) continue;
                const int a[3] = {a0, a1, a2};
                int q[3] = {0, 0, 0};
                T w = 1;
                HG_UNROLL
                for (int d = 0; d < 3; ++d) {
                    if (d >= dm) break;
                    if (odd[d]) w *= (T)0.5;
                    q[d] = node_wrap(G, K, d, lo[d] + a[d]);
                }
                s += w * eK[nix(K, q[0], q[1], q[2])];
            }
    phiF[idx] += s;
}

template <typename T>
HG_HD inline void coarsen_sig_cell(const Geo& G, const LevT<T>& F, const LevT<T>& K, long idx,
                                   T* sK) {
    int c[3];
    cell_coords(K, idx, c);
    const int r0 = G.dm > 0 ? 2 : 1, r1 = G.dm > 1 ? 2 : 1, r2 = G.dm > 2 ? 2 : 1;
    T s = 0;
    for (int c2 = 0; c2 < r2; ++c2)
        for (int c1 = 0; c1 < r1; ++c1)
            for (int c0 = 0; c0 < r0; ++c0)
                s += F.sig[cix(F, c[0] * r0 + c0, c[1] * r1 + c1, c[2] * r2 + c2)];
    sK[idx] = s / (T)(r0 * r1 * r2);
}

// Periodic image nodes take the value of the node they stand for; outflow nodes hold 0.
template <typename T>
HG_HD inline void finish_node(const Geo& G, const LevT<T>& L, long idx, T* x) {
    int p[3];
    node_coords(L, idx, p);
    if (is_unknown(G, L, p)) return;
    int q[3] = {p[0], p[1], p[2]};
    bool fixed = false;
    for (int d = 0; d < G.dm; ++d) {
        if (G.per[d])
            q[d] = node_wrap(G, L, d, p[d]);
        else if ((p[d] == 0 && G.dlo[d]) || (p[d] == L.n[d] && G.dhi[d]))
            fixed = true;
    }
    x[idx] = fixed ? (T)0 : x[nix(L, q[0], q[1], q[2])];
}

// Node-centred divergence of beta0 U (u component-major over the cells; b0 null: 1), minus
// the nodal source (nullable).  Cells outside a non-periodic face carry U = 0, except that at an
// inflow face (W) the cell just outside contributes its wall value of beta0 U_d through the face:
// the boundary flux of the finite-element divergence, with the inflow velocity on the wall.
// The signed sums of beta0 U_d are formed per direction (one FMA a term) and scaled by 1 / h_d
// once: 3 FP64 operations a cell instead of 3 a term, the FP64 pipe being GB300's narrow one.
HG_HD inline void divu_node(const Geo& G, const Lev& L, long idx, const double* u,
                            const double* b0, const double* nodalrhs, const Wall& W, double* rh) {
    int p[3];
    node_coords(L, idx, p);
    const int dm = G.dm;
    const long nc = ncells(L);
    double sd[3] = {0.0, 0.0, 0.0};
    // a node with all 2^dm cells inside and unfolded: direct offsets, the same terms in the same
    // order as the general loop below
    bool inner = true;
    HG_UNROLL
    for (int d = 0; d < 3; ++d) {
        if (d >= dm) break;
        inner = inner && p[d] >= 1 && p[d] <= L.n[d] - 1;
    }
    if (inner) {
        HG_UNROLL
        for (int a = 0; a < 8; ++a) {
            if (a >= (1 << dm)) break;
            const long ci = cix(L, p[0] - (a & 1), dm > 1 ? p[1] - ((a >> 1) & 1) : 0,
                                dm > 2 ? p[2] - ((a >> 2) & 1) : 0);
            const double bb = b0 ? b0[ci] : 1.0;
            HG_UNROLL
            for (int d = 0; d < 3; ++d) {
                if (d >= dm) break;
                sd[d] = fma(((a >> d) & 1) ? -bb : bb, u[d * nc + ci], sd[d]);
            }
        }
    } else {
        HG_UNROLL
        for (int a = 0; a < 8; ++a) {   // (static bounds keep the small arrays in registers)
            if (a >= (1 << dm)) break;
            int c[3] = {0, 0, 0};
            int nout = 0, dout = 0, side = 0;
            HG_UNROLL
            for (int d = 0; d < 3; ++d) {
                if (d >= dm) break;
                const int raw = p[d] - ((a >> d) & 1);
                const int cw = cell_wrap(G, L, d, raw);
                if (cw < 0) {
                    ++nout;
                    dout = d;
                    side = raw < 0 ? 0 : 1;
                }
                c[d] = cw;
            }
            if (nout == 0) {
                const long ci = cix(L, c[0], c[1], c[2]);
                const double bb = b0 ? b0[ci] : 1.0;
                HG_UNROLL
                for (int d = 0; d < 3; ++d) {
                    if (d >= dm) break;
                    sd[d] = fma(((a >> d) & 1) ? -bb : bb, u[d * nc + ci], sd[d]);
                }
            } else if (nout == 1 && W.off[2 * dout + side] >= 0) {
                // the ghost cell just outside an inflow face: its normal velocity is the wall
                // value (its flux through the face), the tangential ones carry no flux out of the
                // domain
                const int e1 = dout == 0 ? 1 : 0;
                const int e2 = dout == 2 ? 1 : 2;
                const long t = c[e1] + (dm == 3 ? (long)L.n[e1] * c[e2] : 0L);
                const double w = W.w[W.off[2 * dout + side] + t];
                HG_UNROLL
                for (int d = 0; d < 3; ++d)
                    if (d == dout) sd[d] += ((a >> d) & 1) ? -w : w;
            }
        }
    }
    double s = sd[0] * L.ih[0];
    HG_UNROLL
    for (int d = 1; d < 3; ++d) {
        if (d >= dm) break;
        s = fma(sd[d], L.ih[d], s);
    }
    s *= 1.0 / (1 << (dm - 1));
    if (nodalrhs) s -= nodalrhs[idx];
    rh[idx] = s;
}

// create_uvec_for_projection (Source/hgproject.f90:437-513) and the solver coefficient of a
// cell: sigma = beta0 / rhohalf (beta0^2 / rhohalf with the alt energy fix outside the initial
// and divu projections).
// 1 / x: on the GPU the FP64 Newton reciprocal of the MAC kernels (recip_nr, within 1 ulp of the
// division and a fraction of its FP64 instructions; the file that launches these functions
// includes mac_internal.cuh first), on the host the division.
HG_HD inline double recip_cell(double x) {
#if defined(__CUDA_ARCH__)
    return recip_nr(x);
#else
    return 1.0 / x;
#endif
}

// idt = 1 / dt, formed once by the caller.
HG_HD inline void uvec_cell(const Geo& G, long idx, long nc, int proj_type, double dt, double idt,
                            double* unew, const double* uold, const double* gpi,
                            const double* rhohalf, const double* b0, int alt, double* sig) {
    // one reciprocal per cell (FP64 division being slow on the GPU): 1 / rhohalf
    const double irho = recip_cell(rhohalf[idx]);
    for (int d = 0; d < G.dm; ++d) {
        double& u = unew[d * nc + idx];
        if (proj_type == kPressureIters) u = (u - uold[d * nc + idx]) * idt;
        else if (proj_type == kRegular) u = u + dt * gpi[d * nc + idx] * irho;
    }
    const double bb = b0 ? b0[idx] : 1.0;
    sig[idx] = (alt ? bb * bb : bb) * irho;
}

// hg_update (Source/hgproject.f90:867-1009) on one cell; gphi written to gpi per proj_type;
// idt = 1 / dt, formed once by the caller.
HG_HD inline void update_cell(const Geo& G, const Lev& L, long idx, int proj_type, double dt,
                              double idt, const double* phi, double* unew, const double* uold,
                              double* gpi, const double* rhohalf, const double* b0, int alt) {
    const long nc = ncells(L);
    // one reciprocal per cell (FP64 division being slow on the GPU): 1 / rhohalf
    const double irho = recip_cell(rhohalf[idx]);
    // mkgphi (Source/hgproject.f90:605-636): gphi_d = 2^(1-dm) [phi summed over the cell's nodes
    // on its + side along d - the same on the - side] / h_d.  The cell's 2^dm nodes are read once
    // for all directions, by direct offsets where no node folds through the periodic wrap.
    int c[3];
    cell_coords(L, idx, c);
    const int dm = G.dm;
    bool inner = true;
    HG_UNROLL
    for (int e = 0; e < 3; ++e) {
        if (e >= dm) break;
        inner = inner && !(G.per[e] && c[e] + 1 >= L.n[e]);
    }
    double pv[8];
    HG_UNROLL
    for (int b = 0; b < 8; ++b) {
        if (b >= (1 << dm)) break;
        int m[3] = {0, 0, 0};
        HG_UNROLL
        for (int e = 0; e < 3; ++e) {
            if (e >= dm) break;
            m[e] = inner ? c[e] + ((b >> e) & 1) : node_wrap(G, L, e, c[e] + ((b >> e) & 1));
        }
        pv[b] = phi[nix(L, m[0], m[1], m[2])];
    }
    for (int d = 0; d < G.dm; ++d) {
        double sg = 0.0;
        HG_UNROLL
        for (int b = 0; b < 8; ++b) {
            if (b >= (1 << dm)) break;
            sg += (((b >> d) & 1) ? 1.0 : -1.0) * pv[b];
        }
        // (2^(1-dm) / h_d as one factor: the power of two scales exactly)
        double g = sg * ((1.0 / (1 << (dm - 1))) * L.ih[d]);
        if (alt) g *= b0 ? b0[idx] : 1.0;
        double& u = unew[d * nc + idx];
        u -= g * irho;
        if (proj_type == kPressureIters) u = uold[d * nc + idx] + dt * u;
        double& gp = gpi[d * nc + idx];
        if (proj_type == kInitial || proj_type == kDivuIters) gp = 0.0;
        else if (proj_type == kPressureIters) gp += g;
        else if (proj_type == kRegular) gp = g * idt;
    }
}

HG_HD inline void update_pi_node(const Lev& L, long idx, int proj_type, double dt,
                                 const double* phi, double* pi) {
    if (proj_type == kInitial || proj_type == kDivuIters) pi[idx] = 0.0;
    else if (proj_type == kPressureIters) pi[idx] += phi[idx];
    else if (proj_type == kRegular) pi[idx] = phi[idx] / dt;
    (void)L;
}

// ---- mixed precision: FP32 inner cycles inside FP64 iterative refinement ---------------------
//
// The FP32 right-hand side of an inner solve is the FP64 defect rounded; the FP64 solution takes
// the FP32 correction on the unknowns; the FP32 coefficients are the FP64 ones rounded.
HG_HD inline void to_single_node(long idx, const double* r, float* r32) { r32[idx] = (float)r[idx]; }
HG_HD inline void accumulate_node(const Geo& G, const Lev& L, long idx, double* phi,
                                  const float* e) {
    int p[3];
    node_coords(L, idx, p);
    if (is_unknown(G, L, p)) phi[idx] += (double)e[idx];
}

// ---- caller fabs <-> whole-domain arrays --------------------------------------------------------
//
// One fab of the caller's layout: box [lo, hi] in cells, ng ghosts, cell- or node-centred
// (nodal: one more entry along every active direction), components of `count` entries each.
struct Fab {
    const double* src;
    double* dst;
    int lo[3], hi[3];
    int ext[3];
    int ng;
    int nodal;
    long count;
};

// Whole-domain index (cells or nodes) of entry e of one component of fab B when it is the box's
// own cell / node, else -1 (ghosts are neither read nor written).
HG_HD inline long fab_target(const Geo& G, const Lev& L, const Fab& B, long e) {
    int a[3];
    a[0] = (int)(e % B.ext[0]);
    const long r = e / B.ext[0];
    a[1] = (int)(r % B.ext[1]);
    a[2] = (int)(r / B.ext[1]);
    int g[3] = {0, 0, 0};
    for (int d = 0; d < G.dm; ++d) {
        g[d] = B.lo[d] - B.ng + a[d];
        if (g[d] < B.lo[d] || g[d] > B.hi[d] + B.nodal) return -1;
    }
    return B.nodal ? nix(L, g[0], g[1], g[2]) : cix(L, g[0], g[1], g[2]);
}

// ---- the nodal V-cycle and the projection -----------------------------------------------------
//
// E provides: int nlev; Geo geo; bool singular; Lev lev(l);
//   double* buf(l, which) node arrays kPhi, kF, kR per level;
//   void defect(l, phi, f, r); void gs(l, phi, f, nu) (nu colour-ordered sweeps);
//   void bottom_gs(l, phi, f, nu) (the same on the coarsest level, one launch on the GPU);
//   void restrict_to(lc, rF, fK) and void prolong(lc, eK, phiF) between levels lc - 1 and lc;
//   void zero(l, x); void finish(l, x); double unknown_max(l, x) (host value);
//   void sub_unknown_mean(l, x) (device-side); int error();
// and for the projection: void uvec(); int build_levels(); void divu(); void update(); level
// 0's buffers hold phi (kPhi) and the right-hand side (kF).
enum { kPhi = 0, kF = 1, kR = 2, kNumBufs = 3 };
constexpr int kBottomSweeps = 60;

template <class E>
void vcycle(E& ex, int l, int nu1, int nu2) {
    if (l == ex.nlev - 1) {
        if (ex.singular) ex.sub_unknown_mean(l, ex.buf(l, kF));
        ex.bottom_gs(l, ex.buf(l, kPhi), ex.buf(l, kF), kBottomSweeps);
        if (ex.singular) ex.sub_unknown_mean(l, ex.buf(l, kPhi));
        return;
    }
    ex.gs(l, ex.buf(l, kPhi), ex.buf(l, kF), nu1);
    ex.defect(l, ex.buf(l, kPhi), ex.buf(l, kF), ex.buf(l, kR));
    ex.restrict_to(l + 1, ex.buf(l, kR), ex.buf(l + 1, kF));
    ex.zero(l + 1, ex.buf(l + 1, kPhi));
    vcycle(ex, l + 1, nu1, nu2);
    ex.prolong(l + 1, ex.buf(l + 1, kPhi), ex.buf(l, kPhi));
    ex.gs(l, ex.buf(l, kPhi), ex.buf(l, kF), nu2);
}

// `count` V-cycles from level 0.  An executor with a member run_cycles(count, nu1, nu2) runs
// them itself (the GPU executor replays a captured CUDA graph of the cycles); otherwise they are
// issued one after the other.
template <class E, class = void>
struct HasRunCycles : std::false_type {};
template <class E>
struct HasRunCycles<E, std::void_t<decltype(std::declval<E&>().run_cycles(0, 0, 0))>>
    : std::true_type {};
template <class E>
void vcycles(E& ex, int count, int nu1, int nu2) {
    if constexpr (HasRunCycles<E>::value) {
        ex.run_cycles(count, nu1, nu2);
    } else {
        for (int v = 0; v < count; ++v) vcycle(ex, 0, nu1, nu2);
    }
}

struct SolveStats {
    int status;
    int cycles;
    double fnorm, resid0, rel_resid;
    int nhist;
    double hist[64];
};

// Solve L phi = f on level 0 from phi = 0 (buf(0, kPhi) zeroed by the caller, f in buf(0, kF)).
// With phi = 0 the defect is f on the unknown nodes, so the first residual norm is fnorm and
// needs no operator pass.
template <class E>
int solve(E& ex, double rel_eps, int max_cycles, int nu1, int nu2, SolveStats* S) {
    *S = SolveStats{};
    if (ex.singular) ex.sub_unknown_mean(0, ex.buf(0, kF));
    const double fnorm = ex.unknown_max(0, ex.buf(0, kF));
    S->fnorm = fnorm;
    if (!(fnorm > 0.0)) {
        ex.zero(0, ex.buf(0, kPhi));
        S->status = std::isnan(fnorm) ? -1 : 0;
        return ex.error() ? ex.error() : S->status;
    }
    double res = fnorm;
    S->resid0 = res;
    int it = 0;
    while (!(res <= rel_eps * fnorm) && it < max_cycles && !std::isnan(res)) {
        vcycles(ex, 1, nu1, nu2);
        ++it;
        ex.defect(0, ex.buf(0, kPhi), ex.buf(0, kF), ex.buf(0, kR));
        res = ex.unknown_max(0, ex.buf(0, kR));
        if (S->nhist < 64) S->hist[S->nhist++] = res / fnorm;
        if (ex.error()) return ex.error();
    }
    S->cycles = it;
    S->rel_resid = res / fnorm;
    S->status = res <= rel_eps * fnorm ? 0 : (std::isnan(res) ? -1 : 1);
    return ex.error() ? ex.error() : S->status;
}

// hgproject on one level with the caller's arrays loaded in the executor.
template <class E>
int project(E& ex, double rel_eps, int max_cycles, int nu1, int nu2, SolveStats* S) {
    ex.uvec();                   // U per proj_type, sigma of level 0
    int rc = ex.build_levels();  // coarse sigma
    if (rc) return rc;
    ex.divu();                   // buf(0, kF) = D(beta0 U) - nodalrhs
    ex.zero(0, ex.buf(0, kPhi));
    rc = solve(ex, rel_eps, max_cycles, nu1, nu2, S);
    if (rc < 0) return rc;
    const int status = rc;
    ex.finish(0, ex.buf(0, kPhi));
    ex.update();                 // U, gpi, pi
    rc = ex.error();
    return rc ? rc : status;
}

// Mixed-precision solve from phi = 0: FP64 defect, `inner` FP32 V-cycles on it from zero (ex32:
// the FP32 view of the same hierarchy), FP64 accumulation, until the FP64 residual meets rel_eps.
template <class E, class E32>
int solve_mixed(E& ex, E32& ex32, double rel_eps, int max_iters, int nu1, int nu2, int inner,
                SolveStats* S) {
    *S = SolveStats{};
    if (ex.singular) ex.sub_unknown_mean(0, ex.buf(0, kF));
    const double fnorm = ex.unknown_max(0, ex.buf(0, kF));
    S->fnorm = fnorm;
    if (!(fnorm > 0.0)) {
        ex.zero(0, ex.buf(0, kPhi));
        S->status = std::isnan(fnorm) ? -1 : 0;
        return ex.error() ? ex.error() : S->status;
    }
    // phi = 0: the first defect is f on the unknown nodes (the FP32 cycles read their right-hand
    // side on unknown nodes only), and its norm is fnorm
    double res = fnorm;
    S->resid0 = res;
    int it = 0;
    while (!(res <= rel_eps * fnorm) && it < max_iters && !std::isnan(res)) {
        ex.to_single(ex.buf(0, it == 0 ? kF : kR), ex32.buf(0, kF));
        ex32.zero(0, ex32.buf(0, kPhi));
        vcycles(ex32, inner, nu1, nu2);
        ex.accumulate(ex.buf(0, kPhi), ex32.buf(0, kPhi));
        ex.defect(0, ex.buf(0, kPhi), ex.buf(0, kF), ex.buf(0, kR));
        res = ex.unknown_max(0, ex.buf(0, kR));
        ++it;
        if (S->nhist < 64) S->hist[S->nhist++] = res / fnorm;
        if (ex.error() || ex32.error()) return ex.error() ? ex.error() : ex32.error();
    }
    S->cycles = it * inner;
    S->rel_resid = res / fnorm;
    S->status = res <= rel_eps * fnorm ? 0 : (std::isnan(res) ? -1 : 1);
    return ex.error() ? ex.error() : S->status;
}

// hgproject with the mixed-precision solve.
template <class E, class E32>
int project_mixed(E& ex, E32& ex32, double rel_eps, int max_iters, int nu1, int nu2, int inner,
                  SolveStats* S) {
    ex.uvec();
    int rc = ex.build_levels();
    if (rc) return rc;
    ex.sig_to_single();   // FP32 coefficients of every level
    ex.divu();
    ex.zero(0, ex.buf(0, kPhi));
    rc = solve_mixed(ex, ex32, rel_eps, max_iters, nu1, nu2, inner, S);
    if (rc < 0) return rc;
    const int status = rc;
    ex.finish(0, ex.buf(0, kPhi));
    ex.update();
    rc = ex.error();
    return rc ? rc : status;
}

}  // namespace hg
}  // namespace mac
