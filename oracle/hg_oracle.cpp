// Nodal (HG) projection oracle: a CPU (C++17 + OpenMP, IEEE FP64) restatement of MAESTRO's
// `hgproject` on one level and of the FBoxLib nodal multigrid solve `hg_multigrid` hands it to.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product path may link, load or call it.
//
// What it follows (paths are within the MAESTRO source tree):
//   Source/hgproject.f90:32-264     hgproject: create_uvec_for_projection, U *= beta0,
//                                   rhohalf /= beta0 (twice with the alt energy fix outside the
//                                   initial and divu projections), the nodal solve, U /= beta0,
//                                   rhohalf *= beta0, mkgphi, hg_update
//   Source/hgproject.f90:437-513    create_uvec_3d per proj_type; wall ghost cells of U set to 0
//   Source/hgproject.f90:605-636    mkgphi_3d: cell gradient = mean of the nodal differences
//   Source/hgproject.f90:867-1009   hg_update_3d: U -= gphi / rhohalf (gphi *= beta0 with the
//                                   alt energy fix), pi / gpi per proj_type
//   Source/hg_multigrid.f90:18-239  coefficients 1 / rhohalf on the valid cells, 0 in ghost
//                                   cells; divu; rh -= nodalrhs; ml_nd_solve
//   Source/mg_eps.f90:23-31         eps_hg = 1e-12, eps_hg_bottom = 1e-4
//   Docs/mg/mg.tex:379-500          nodal MG (restriction, prolongation), the node-centred
//                                   divergence, dense (9/27-point) and cross (5/7-point) stencils
//
// FBoxLib is not part of the MAESTRO tree; the nodal arithmetic is written from that description
// and the mathematics:
//   * nodes     : (n_d + 1) per direction in storage; periodic directions identify node n_d with
//                 node 0; nodes on an outflow (Dirichlet) face are fixed at 0.
//   * divergence: DU_p = sum_d (1/h_d) 2^(1-dm) [sum of u_d over the cells on the + side of p -
//                 the same on the - side] (Docs/mg/mg.tex:485-493); cells outside a non-periodic
//                 face carry U = 0 (create_uvec sets wall ghosts to 0), except that the ghost
//                 cell outside an inlet face adds the flux of its normal velocity (orc_hg_opts
//                 wall: the inflow on the wall, lo_inflow / hi_inflow of hg_multigrid).
//   * dense     : the bilinear / trilinear finite-element stiffness per cell, scaled by the cell
//                 coefficient sigma and divided by the nodal volume prod h_d:
//                 (L phi)_p = - sum_{cells c of p} sigma_c sum_{nodes m of c} sum_d h_d^-2
//                             S(p_d, m_d) prod_{e != d} M(p_e, m_e) phi_m,
//                 S = [[1,-1],[-1,1]], M = [[1/3,1/6],[1/6,1/3]] (local 0/1 positions in c);
//                 sigma = 0 outside non-periodic faces.
//   * cross     : (L phi)_p = sum_d h_d^-2 sum_s sigma_e (phi_{p + s e_d} - phi_p), sigma_e the
//                 mean of sigma over the 2^(dm-1) cells along the edge (0 outside the domain).
//   * solve     : L phi = DU - nodalrhs, V(2,2)-cycles, 2^dm-colour Gauss-Seidel (node parity),
//                 full-weighting restriction of the defect, multilinear prolongation (coincident
//                 nodes copied), coarse sigma = mean of the fine cells, Jacobi-preconditioned CG
//                 to eps_hg_bottom on the coarsest level; singular problem (no outflow face): the
//                 mean of the right-hand side over the unknown nodes removed.  Converged when
//                 max |rh - L phi| <= eps max |rh| over the unknown nodes.
//   * gradient  : gphi_d(c) = 2^(1-dm) [sum of phi over the nodes of c on its + side along d - the
//                 same on the - side] / h_d (mkgphi).

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mac_oracle_core.h"

extern "C" {

enum { HG_INITIAL = 1, HG_DIVU_ITERS = 2, HG_PRESSURE_ITERS = 3, HG_REGULAR = 4 };

typedef struct orc_hg_opts {
    int dm;
    int n[3];            // cells
    double dx[3];
    int bc_lo[3];        // ORC_BC_PER / ORC_BC_NEU (walls, inflow, symmetry) / ORC_BC_DIR (outflow)
    int bc_hi[3];
    int dense;           // 1: dense stencil (hg_dense_stencil), 0: cross
    int proj_type;       // HG_*
    double dt;
    int alt_energy_fix;
    double rel_eps;
    int max_vcycles;
    int nu1, nu2;
    double bottom_eps;
    int nthreads;
    // inflow (inlet) faces: face f = 2 d + side (0 low, 1 high) is an inlet when wall_off[f] >= 0;
    // wall + wall_off[f] then holds, for each cell of the face (its other directions, Fortran
    // order), the wall value of beta0 U_d the ghost cell outside it carries
    long wall_off[6];
    const double* wall;
} orc_hg_opts;

}  // extern "C"

namespace {

using std::size_t;

struct NLev {
    int n[3];       // cells
    double h[3];
    std::vector<double> sig;   // cells
    std::vector<double> phi, f, r;   // nodes (n+1 per active direction)
    int nn[3];      // node storage extents
    size_t nnodes() const { return (size_t)nn[0] * nn[1] * nn[2]; }
    size_t ncells() const { return (size_t)n[0] * n[1] * n[2]; }
};

struct NCtx {
    orc_hg_opts o;
    int dm;
    std::vector<NLev> lev;
    bool singular;
};

inline size_t nidx(const NLev& L, int i, int j, int k) {
    return (size_t)i + (size_t)L.nn[0] * ((size_t)j + (size_t)L.nn[1] * k);
}
inline size_t cidx3(const NLev& L, int i, int j, int k) {
    return (size_t)i + (size_t)L.n[0] * ((size_t)j + (size_t)L.n[1] * k);
}

// Node index q along d folded onto storage (periodic: n -> 0, wrap); -1 outside.
inline int node_wrap(const NCtx& C, const NLev& L, int d, int q) {
    const int n = L.n[d];
    if (d >= C.dm) return q == 0 ? 0 : -1;
    if (C.o.bc_lo[d] == ORC_BC_PER) return ((q % n) + n) % n;
    return (q < 0 || q > n) ? -1 : q;
}
// Cell index c along d (periodic wrap); -1 outside.
inline int cell_wrap(const NCtx& C, const NLev& L, int d, int c) {
    const int n = L.n[d];
    if (d >= C.dm) return c == 0 ? 0 : -1;
    if (C.o.bc_lo[d] == ORC_BC_PER) return ((c % n) + n) % n;
    return (c < 0 || c >= n) ? -1 : c;
}
// Whether storage node p is an unknown (not a periodic image, not on an outflow face).
inline bool is_unknown(const NCtx& C, const NLev& L, const int p[3]) {
    for (int d = 0; d < C.dm; ++d) {
        if (C.o.bc_lo[d] == ORC_BC_PER) {
            if (p[d] == L.n[d]) return false;
        } else {
            if (p[d] == 0 && C.o.bc_lo[d] == ORC_BC_DIR) return false;
            if (p[d] == L.n[d] && C.o.bc_hi[d] == ORC_BC_DIR) return false;
        }
    }
    return true;
}

const double kM[2][2] = {{1.0 / 3.0, 1.0 / 6.0}, {1.0 / 6.0, 1.0 / 3.0}};
const double kS[2][2] = {{1.0, -1.0}, {-1.0, 1.0}};

// (L phi)_p split into diag * phi_p - off.
void node_op(const NCtx& C, const NLev& L, const int p[3], const double* phi, double& diag,
             double& off) {
    const int dm = C.dm;
    diag = 0.0;
    off = 0.0;
    const size_t pi = nidx(L, p[0], p[1], p[2]);
    if (C.o.dense) {
        for (int a = 0; a < (1 << dm); ++a) {
            int c[3] = {0, 0, 0}, loc[3] = {0, 0, 0};
            bool out = false;
            for (int d = 0; d < dm; ++d) {
                loc[d] = (a >> d) & 1;   // local position of p in the cell: 1 = p is its + corner
                const int cw = cell_wrap(C, L, d, p[d] - loc[d]);
                if (cw < 0) out = true;
                c[d] = cw;
            }
            if (out) continue;
            const double s = L.sig[cidx3(L, c[0], c[1], c[2])];
            for (int b = 0; b < (1 << dm); ++b) {
                int m[3] = {0, 0, 0}, ml[3] = {0, 0, 0};
                for (int d = 0; d < dm; ++d) {
                    ml[d] = (b >> d) & 1;
                    m[d] = node_wrap(C, L, d, c[d] + ml[d]);
                }
                double k = 0.0;
                for (int d = 0; d < dm; ++d) {
                    double t = kS[loc[d]][ml[d]] / (L.h[d] * L.h[d]);
                    for (int e = 0; e < dm; ++e)
                        if (e != d) t *= kM[loc[e]][ml[e]];
                    k += t;
                }
                const size_t mi = nidx(L, m[0], m[1], m[2]);
                if (mi == pi)
                    diag += s * k;
                else
                    off -= s * k * phi[mi];
            }
        }
        // L phi = -(K phi): diag_L = -sum k (negative), off as the other side
        diag = -diag;
        off = -off;
        // now L phi = diag * phi_p - off  with diag < 0
    } else {
        for (int d = 0; d < dm; ++d) {
            for (int sd = -1; sd <= 1; sd += 2) {
                const int q = node_wrap(C, L, d, p[d] + sd);
                if (q < 0) continue;
                // cells along the edge p -> p + sd e_d: index min(p_d, p_d + sd) along d, the
                // 2^(dm-1) cells around the edge in the other directions
                double sum = 0.0;
                int cnt = 0;
                for (int a = 0; a < (1 << dm); ++a) {
                    if ((a >> d) & 1) continue;
                    int c[3] = {0, 0, 0};
                    bool out = false;
                    for (int e = 0; e < dm; ++e) {
                        const int want = e == d ? std::min(p[d], p[d] + sd) : p[e] - ((a >> e) & 1);
                        const int cw = cell_wrap(C, L, e, want);
                        if (cw < 0) out = true;
                        c[e] = cw;
                    }
                    ++cnt;
                    if (!out) sum += L.sig[cidx3(L, c[0], c[1], c[2])];
                }
                const double se = sum / cnt / (L.h[d] * L.h[d]);
                int qq[3] = {p[0], p[1], p[2]};
                qq[d] = q;
                diag -= se;
                off -= se * phi[nidx(L, qq[0], qq[1], qq[2])];
            }
        }
        // L phi = sum se (phi_q - phi_p) = diag * phi_p - off with diag = -sum se, off = -sum se phi_q
    }
}

double resid(const NCtx& C, const NLev& L, const double* phi, const double* f, double* r) {
    double mx = 0.0;
#pragma omp parallel for schedule(static) reduction(max : mx)
    for (int k = 0; k < L.nn[2]; ++k)
        for (int j = 0; j < L.nn[1]; ++j)
            for (int i = 0; i < L.nn[0]; ++i) {
                const int p[3] = {i, j, k};
                const size_t pi = nidx(L, i, j, k);
                if (!is_unknown(C, L, p)) {
                    if (r) r[pi] = 0.0;
                    continue;
                }
                double dg, off;
                node_op(C, L, p, phi, dg, off);
                const double v = f[pi] - (dg * phi[pi] - off);
                if (r) r[pi] = v;
                mx = std::max(mx, std::fabs(v));
            }
    return mx;
}

// Copy periodic images (node n_d = node 0) so the storage stays consistent.
void sync_images(const NCtx& C, NLev& L, std::vector<double>& x) {
    for (int d = 0; d < C.dm; ++d) {
        if (C.o.bc_lo[d] != ORC_BC_PER) continue;
        for (int k = 0; k < L.nn[2]; ++k)
            for (int j = 0; j < L.nn[1]; ++j)
                for (int i = 0; i < L.nn[0]; ++i) {
                    int p[3] = {i, j, k};
                    if (p[d] != L.n[d]) continue;
                    int q[3] = {i, j, k};
                    for (int e = 0; e < C.dm; ++e)
                        if (C.o.bc_lo[e] == ORC_BC_PER && q[e] == L.n[e]) q[e] = 0;
                    x[nidx(L, p[0], p[1], p[2])] = x[nidx(L, q[0], q[1], q[2])];
                }
    }
}

void smooth(const NCtx& C, NLev& L, int nu) {
    const int dm = C.dm;
    // an odd periodic extent couples same-colour nodes across the wrap: sweep serially then
    bool par = true;
    for (int d = 0; d < dm; ++d) par = par && !(C.o.bc_lo[d] == ORC_BC_PER && (L.n[d] & 1));
    for (int it = 0; it < nu; ++it)
        for (int colour = 0; colour < (1 << dm); ++colour) {
#pragma omp parallel for schedule(static) if (par)
            for (int k = 0; k < L.nn[2]; ++k)
                for (int j = 0; j < L.nn[1]; ++j)
                    for (int i = 0; i < L.nn[0]; ++i) {
                        const int p[3] = {i, j, k};
                        int col = 0;
                        for (int d = 0; d < dm; ++d) col |= (p[d] & 1) << d;
                        if (col != colour || !is_unknown(C, L, p)) continue;
                        double dg, off;
                        node_op(C, L, p, L.phi.data(), dg, off);
                        const size_t pi = nidx(L, i, j, k);
                        L.phi[pi] = (L.f[pi] + off) / dg;
                    }
            sync_images(C, L, L.phi);
        }
}

double mean_unknown(const NCtx& C, const NLev& L, const std::vector<double>& x) {
    double s = 0.0;
    long cnt = 0;
    for (int k = 0; k < L.nn[2]; ++k)
        for (int j = 0; j < L.nn[1]; ++j)
            for (int i = 0; i < L.nn[0]; ++i) {
                const int p[3] = {i, j, k};
                if (!is_unknown(C, L, p)) continue;
                s += x[nidx(L, i, j, k)];
                ++cnt;
            }
    return cnt ? s / cnt : 0.0;
}

void sub_unknown(const NCtx& C, NLev& L, std::vector<double>& x, double m) {
    for (int k = 0; k < L.nn[2]; ++k)
        for (int j = 0; j < L.nn[1]; ++j)
            for (int i = 0; i < L.nn[0]; ++i) {
                const int p[3] = {i, j, k};
                if (is_unknown(C, L, p)) x[nidx(L, i, j, k)] -= m;
            }
    sync_images(C, L, x);
}

// Jacobi-preconditioned CG on the coarsest level (L is symmetric negative semi-definite: solve
// -L phi = -f).
void bottom_cg(NCtx& C, NLev& L) {
    const size_t N = L.nnodes();
    if (C.singular) sub_unknown(C, L, L.f, mean_unknown(C, L, L.f));
    std::vector<double> r(N), z(N), p(N), q(N), dg(N, 1.0);
    for (int k = 0; k < L.nn[2]; ++k)
        for (int j = 0; j < L.nn[1]; ++j)
            for (int i = 0; i < L.nn[0]; ++i) {
                const int pp[3] = {i, j, k};
                if (!is_unknown(C, L, pp)) continue;
                double d, off;
                node_op(C, L, pp, L.phi.data(), d, off);
                dg[nidx(L, i, j, k)] = -d;
            }
    auto apply = [&](const std::vector<double>& x, std::vector<double>& y) {
        std::vector<double> xs = x;
        sync_images(C, L, xs);
        for (int k = 0; k < L.nn[2]; ++k)
            for (int j = 0; j < L.nn[1]; ++j)
                for (int i = 0; i < L.nn[0]; ++i) {
                    const int pp[3] = {i, j, k};
                    const size_t pi = nidx(L, i, j, k);
                    if (!is_unknown(C, L, pp)) {
                        y[pi] = 0.0;
                        continue;
                    }
                    double d, off;
                    node_op(C, L, pp, xs.data(), d, off);
                    y[pi] = -(d * xs[pi] - off);
                }
    };
    auto dot = [&](const std::vector<double>& a, const std::vector<double>& b) {
        double s = 0.0;
        for (int k = 0; k < L.nn[2]; ++k)
            for (int j = 0; j < L.nn[1]; ++j)
                for (int i = 0; i < L.nn[0]; ++i) {
                    const int pp[3] = {i, j, k};
                    if (is_unknown(C, L, pp)) s += a[nidx(L, i, j, k)] * b[nidx(L, i, j, k)];
                }
        return s;
    };
    const double r0 = resid(C, L, L.phi.data(), L.f.data(), r.data());
    if (r0 == 0.0) return;
    for (size_t q2 = 0; q2 < N; ++q2) r[q2] = -r[q2];   // residual of -L phi = -f
    for (size_t q2 = 0; q2 < N; ++q2) z[q2] = r[q2] / dg[q2];
    if (C.singular) sub_unknown(C, L, z, mean_unknown(C, L, z));
    p = z;
    double rz = dot(r, z);
    for (int it = 0; it < 1000 && rz != 0.0; ++it) {
        apply(p, q);
        const double pq = dot(p, q);
        if (pq == 0.0) break;
        const double alpha = rz / pq;
        for (size_t q2 = 0; q2 < N; ++q2) {
            L.phi[q2] += alpha * p[q2];
            r[q2] -= alpha * q[q2];
        }
        double rm = 0.0;
        for (size_t q2 = 0; q2 < N; ++q2) rm = std::max(rm, std::fabs(r[q2]));
        if (rm <= C.o.bottom_eps * r0) break;
        for (size_t q2 = 0; q2 < N; ++q2) z[q2] = r[q2] / dg[q2];
        if (C.singular) sub_unknown(C, L, z, mean_unknown(C, L, z));
        const double rz2 = dot(r, z);
        const double beta = rz2 / rz;
        rz = rz2;
        for (size_t q2 = 0; q2 < N; ++q2) p[q2] = z[q2] + beta * p[q2];
    }
    sync_images(C, L, L.phi);
}

void restrict_fw(const NCtx& C, const NLev& F, NLev& K) {
    const int dm = C.dm;
    std::fill(K.f.begin(), K.f.end(), 0.0);
    for (int k = 0; k < K.nn[2]; ++k)
        for (int j = 0; j < K.nn[1]; ++j)
            for (int i = 0; i < K.nn[0]; ++i) {
                const int P[3] = {i, j, k};
                if (!is_unknown(C, K, P)) continue;
                double s = 0.0;
                for (int a2 = -(dm > 2); a2 <= (dm > 2); ++a2)
                    for (int a1 = -(dm > 1); a1 <= (dm > 1); ++a1)
                        for (int a0 = -1; a0 <= 1; ++a0) {
                            const int a[3] = {a0, a1, a2};
                            int q[3];
                            double w = 1.0;
                            bool out = false;
                            for (int d = 0; d < 3; ++d) {
                                if (d >= dm) {
                                    q[d] = 0;
                                    continue;
                                }
                                w *= a[d] ? 0.5 : 1.0;
                                const int qq = node_wrap(C, F, d, 2 * P[d] + a[d]);
                                if (qq < 0) out = true;
                                q[d] = qq;
                            }
                            if (out) continue;
                            s += w * F.r[nidx(F, q[0], q[1], q[2])];
                        }
                K.f[nidx(K, i, j, k)] = s / (1 << dm);
            }
    sync_images(C, K, K.f);
}

void prolong_add(const NCtx& C, const NLev& K, NLev& F) {
    const int dm = C.dm;
    for (int k = 0; k < F.nn[2]; ++k)
        for (int j = 0; j < F.nn[1]; ++j)
            for (int i = 0; i < F.nn[0]; ++i) {
                const int p[3] = {i, j, k};
                if (!is_unknown(C, F, p)) continue;
                double s = 0.0;
                int lo[3], odd[3];
                for (int d = 0; d < 3; ++d) {
                    lo[d] = d < dm ? p[d] >> 1 : 0;
                    odd[d] = d < dm ? (p[d] & 1) : 0;
                }
                for (int a2 = 0; a2 <= odd[2]; ++a2)
                    for (int a1 = 0; a1 <= odd[1]; ++a1)
                        for (int a0 = 0; a0 <= odd[0]; ++a0) {
                            const int a[3] = {a0, a1, a2};
                            int q[3];
                            double w = 1.0;
                            for (int d = 0; d < 3; ++d) {
                                if (d >= dm) {
                                    q[d] = 0;
                                    continue;
                                }
                                if (odd[d]) w *= 0.5;
                                q[d] = node_wrap(C, K, d, lo[d] + a[d]);
                            }
                            s += w * K.phi[nidx(K, q[0], q[1], q[2])];
                        }
                F.phi[nidx(F, i, j, k)] += s;
            }
    sync_images(C, F, F.phi);
}

void vcycle(NCtx& C, int l) {
    NLev& L = C.lev[l];
    if (l + 1 == (int)C.lev.size()) {
        bottom_cg(C, L);
        return;
    }
    smooth(C, L, C.o.nu1);
    resid(C, L, L.phi.data(), L.f.data(), L.r.data());
    NLev& K = C.lev[l + 1];
    restrict_fw(C, L, K);
    std::fill(K.phi.begin(), K.phi.end(), 0.0);
    vcycle(C, l + 1);
    prolong_add(C, K, L);
    smooth(C, L, C.o.nu2);
}

void build_levels(NCtx& C, const double* sigma) {
    const orc_hg_opts& o = C.o;
    C.dm = o.dm;
    C.lev.clear();
    NLev F;
    for (int d = 0; d < 3; ++d) {
        F.n[d] = d < o.dm ? o.n[d] : 1;
        F.h[d] = o.dx[d];
        F.nn[d] = d < o.dm ? o.n[d] + 1 : 1;
    }
    F.sig.assign(sigma, sigma + F.ncells());
    C.lev.push_back(F);
    while (true) {
        const NLev& P = C.lev.back();
        bool ok = true;
        for (int d = 0; d < o.dm; ++d) ok = ok && P.n[d] % 2 == 0 && P.n[d] >= 4;
        if (!ok) break;
        NLev K;
        for (int d = 0; d < 3; ++d) {
            K.n[d] = d < o.dm ? P.n[d] / 2 : 1;
            K.h[d] = d < o.dm ? P.h[d] * 2 : P.h[d];
            K.nn[d] = d < o.dm ? K.n[d] + 1 : 1;
        }
        K.sig.assign(K.ncells(), 0.0);
        const int r[3] = {o.dm > 0 ? 2 : 1, o.dm > 1 ? 2 : 1, o.dm > 2 ? 2 : 1};
        for (int k = 0; k < K.n[2]; ++k)
            for (int j = 0; j < K.n[1]; ++j)
                for (int i = 0; i < K.n[0]; ++i) {
                    double s = 0.0;
                    for (int c2 = 0; c2 < r[2]; ++c2)
                        for (int c1 = 0; c1 < r[1]; ++c1)
                            for (int c0 = 0; c0 < r[0]; ++c0)
                                s += P.sig[cidx3(P, i * r[0] + c0, j * r[1] + c1, k * r[2] + c2)];
                    K.sig[cidx3(K, i, j, k)] = s / (r[0] * r[1] * r[2]);
                }
        C.lev.push_back(K);
    }
    for (NLev& L : C.lev) {
        L.phi.assign(L.nnodes(), 0.0);
        L.f.assign(L.nnodes(), 0.0);
        L.r.assign(L.nnodes(), 0.0);
    }
    bool dir = false;
    for (int d = 0; d < o.dm; ++d) dir = dir || o.bc_lo[d] == ORC_BC_DIR || o.bc_hi[d] == ORC_BC_DIR;
    C.singular = !dir;
}

int nodal_solve(NCtx& C, const double* rh, double* phi, orc_stats* st) {
    NLev& F = C.lev[0];
    F.f.assign(rh, rh + F.nnodes());
    F.phi.assign(phi, phi + F.nnodes());
    sync_images(C, F, F.f);
    sync_images(C, F, F.phi);
    for (int k = 0; k < F.nn[2]; ++k)   // fixed (outflow) nodes hold 0
        for (int j = 0; j < F.nn[1]; ++j)
            for (int i = 0; i < F.nn[0]; ++i) {
                const int p[3] = {i, j, k};
                bool fixed = false;
                for (int d = 0; d < C.dm; ++d)
                    fixed = fixed || (C.o.bc_lo[d] == ORC_BC_DIR && p[d] == 0) ||
                            (C.o.bc_hi[d] == ORC_BC_DIR && p[d] == F.n[d]);
                if (fixed) F.phi[nidx(F, i, j, k)] = 0.0;
            }
    if (C.singular) sub_unknown(C, F, F.f, mean_unknown(C, F, F.f));
    double fnorm = 0.0;
    for (int k = 0; k < F.nn[2]; ++k)
        for (int j = 0; j < F.nn[1]; ++j)
            for (int i = 0; i < F.nn[0]; ++i) {
                const int p[3] = {i, j, k};
                if (is_unknown(C, F, p)) fnorm = std::max(fnorm, std::fabs(F.f[nidx(F, i, j, k)]));
            }
    orc_stats local{};
    orc_stats& S = st ? *st : local;
    std::memset(&S, 0, sizeof(S));
    S.fnorm = fnorm;
    if (fnorm == 0.0) {
        std::fill(F.phi.begin(), F.phi.end(), 0.0);
        std::copy(F.phi.begin(), F.phi.end(), phi);
        return 0;
    }
    double res = resid(C, F, F.phi.data(), F.f.data(), nullptr);
    S.resid0 = res;
    int it = 0;
    while (!(res <= C.o.rel_eps * fnorm) && it < C.o.max_vcycles) {
        vcycle(C, 0);
        ++it;
        res = resid(C, F, F.phi.data(), F.f.data(), nullptr);
        if (S.nhist < 64) S.hist[S.nhist++] = res / fnorm;
    }
    S.vcycles = it;
    S.rel_resid = res / fnorm;
    S.status = res <= C.o.rel_eps * fnorm ? 0 : 1;
    std::copy(F.phi.begin(), F.phi.end(), phi);
    return S.status;
}

// Node-centred divergence of the cell field u (dm components, component-major), U = 0 in cells
// outside non-periodic faces.  Inflow faces (hg_multigrid's lo_inflow / hi_inflow,
// Source/hg_multigrid.f90:191-204): the ghost cell just outside the face contributes the normal
// component it carries, the inflow velocity on the wall, i.e. the flux through the face; its
// tangential components move nothing out of the domain.  (FBoxLib's divu is not in the MAESTRO
// tree; this is the finite-element divergence with the prescribed boundary flux.)
void nodal_divu(const NCtx& C, const NLev& L, const double* u, double* out) {
    const int dm = C.dm;
    const size_t nc = L.ncells();
    for (int k = 0; k < L.nn[2]; ++k)
        for (int j = 0; j < L.nn[1]; ++j)
            for (int i = 0; i < L.nn[0]; ++i) {
                const int p[3] = {i, j, k};
                double s = 0.0;
                for (int a = 0; a < (1 << dm); ++a) {
                    int c[3] = {0, 0, 0};
                    int nout = 0, dout = -1, side = 0;
                    for (int d = 0; d < dm; ++d) {
                        const int raw = p[d] - ((a >> d) & 1);
                        const int cw = cell_wrap(C, L, d, raw);
                        if (cw < 0) {
                            ++nout;
                            dout = d;
                            side = raw < 0 ? 0 : 1;
                        }
                        c[d] = cw;
                    }
                    if (nout == 0) {
                        const size_t ci = cidx3(L, c[0], c[1], c[2]);
                        for (int d = 0; d < dm; ++d) {
                            const double sgn = ((a >> d) & 1) ? -1.0 : 1.0;   // cell on the - side
                            s += sgn * u[d * nc + ci] / L.h[d];
                        }
                    } else if (nout == 1 && C.o.wall && C.o.wall_off[2 * dout + side] >= 0) {
                        // index of the ghost cell within the face: the other directions in order
                        size_t t = 0, stride = 1;
                        for (int e = 0; e < dm; ++e) {
                            if (e == dout) continue;
                            t += stride * (size_t)c[e];
                            stride *= (size_t)L.n[e];
                        }
                        const double sgn = ((a >> dout) & 1) ? -1.0 : 1.0;
                        s += sgn * C.o.wall[C.o.wall_off[2 * dout + side] + t] / L.h[dout];
                    }
                }
                out[nidx(L, i, j, k)] = s / (1 << (dm - 1));
            }
}

// mkgphi: cell gradient of the nodal phi.
void nodal_grad(const NCtx& C, const NLev& L, const double* phi, double* g) {
    const int dm = C.dm;
    const size_t nc = L.ncells();
    for (int k = 0; k < L.n[2]; ++k)
        for (int j = 0; j < L.n[1]; ++j)
            for (int i = 0; i < L.n[0]; ++i) {
                const int c[3] = {i, j, k};
                for (int d = 0; d < dm; ++d) {
                    double s = 0.0;
                    for (int b = 0; b < (1 << dm); ++b) {
                        int m[3] = {0, 0, 0};
                        for (int e = 0; e < dm; ++e) m[e] = node_wrap(C, L, e, c[e] + ((b >> e) & 1));
                        s += (((b >> d) & 1) ? 1.0 : -1.0) * phi[nidx(L, m[0], m[1], m[2])];
                    }
                    g[d * nc + cidx3(L, i, j, k)] = s / (1 << (dm - 1)) / L.h[d];
                }
            }
}

}  // namespace

extern "C" {

// Nodal operator L phi (cells -> sigma, nodes phi -> out), for the pin tests.
void orc_hg_apply(const orc_hg_opts* o, const double* sigma, const double* phi, double* out) {
    NCtx C;
    C.o = *o;
    build_levels(C, sigma);
    NLev& F = C.lev[0];
    std::vector<double> zero(F.nnodes(), 0.0);
    resid(C, F, phi, zero.data(), out);
    for (size_t q = 0; q < F.nnodes(); ++q) out[q] = -out[q];
}

// Node-centred divergence of a cell vector field (component-major, dm components).
void orc_hg_divu(const orc_hg_opts* o, const double* u, double* out) {
    NCtx C;
    C.o = *o;
    std::vector<double> one((size_t)o->n[0] * (o->dm > 1 ? o->n[1] : 1) * (o->dm > 2 ? o->n[2] : 1), 1.0);
    build_levels(C, one.data());
    nodal_divu(C, C.lev[0], u, out);
}

// Cell gradient of a nodal field (mkgphi).
void orc_hg_grad(const orc_hg_opts* o, const double* phi, double* g) {
    NCtx C;
    C.o = *o;
    std::vector<double> one((size_t)o->n[0] * (o->dm > 1 ? o->n[1] : 1) * (o->dm > 2 ? o->n[2] : 1), 1.0);
    build_levels(C, one.data());
    nodal_grad(C, C.lev[0], phi, g);
}

// Solve L phi = rh on the nodes with cell coefficients sigma; phi in/out.
int orc_hg_solve(const orc_hg_opts* o, const double* sigma, const double* rh, double* phi,
                 orc_stats* st) {
#ifdef _OPENMP
    if (o->nthreads > 0) omp_set_num_threads(o->nthreads);
#endif
    NCtx C;
    C.o = *o;
    build_levels(C, sigma);
    return nodal_solve(C, rh, phi, st);
}

// hgproject on one level (Source/hgproject.f90:32-264).  Cell arrays (n0, n1[, n2]) in Fortran
// order: unew / uold / gpi with dm components (component-major), rhohalf, beta0 (beta0_cart;
// nullable: 1).  Node arrays (n0+1, n1+1[, n2+1]): pi (in/out), nodalrhs (nullable).  phi_out
// (nullable) receives the nodal solution.  Returns the solve status.
int orc_hgproject(const orc_hg_opts* o, double* unew, const double* uold, double* gpi,
                  const double* rhohalf_in, double* pi, const double* beta0,
                  const double* nodalrhs, double* phi_out, orc_stats* st) {
#ifdef _OPENMP
    if (o->nthreads > 0) omp_set_num_threads(o->nthreads);
#endif
    const int dm = o->dm;
    NCtx C;
    C.o = *o;
    const size_t nc = (size_t)o->n[0] * (dm > 1 ? o->n[1] : 1) * (dm > 2 ? o->n[2] : 1);
    std::vector<double> rhoh(rhohalf_in, rhohalf_in + nc);
    // create_uvec_for_projection
    for (int d = 0; d < dm; ++d)
        for (size_t c = 0; c < nc; ++c) {
            double& u = unew[d * nc + c];
            if (o->proj_type == HG_PRESSURE_ITERS) u = (u - uold[d * nc + c]) / o->dt;
            else if (o->proj_type == HG_REGULAR) u = u + o->dt * gpi[d * nc + c] / rhoh[c];
        }
    const bool alt = o->proj_type != HG_INITIAL && o->proj_type != HG_DIVU_ITERS && o->alt_energy_fix;
    for (size_t c = 0; c < nc; ++c) {
        const double b = beta0 ? beta0[c] : 1.0;
        for (int d = 0; d < dm; ++d) unew[d * nc + c] *= b;
        rhoh[c] /= b;
        if (alt) rhoh[c] /= b;
    }
    std::vector<double> sigma(nc);
    for (size_t c = 0; c < nc; ++c) sigma[c] = 1.0 / rhoh[c];
    build_levels(C, sigma.data());
    NLev& F = C.lev[0];
    const size_t nn = F.nnodes();
    std::vector<double> rh(nn), phi(nn, 0.0);
    nodal_divu(C, F, unew, rh.data());
    if (nodalrhs)
        for (size_t q = 0; q < nn; ++q) rh[q] -= nodalrhs[q];
    const int status = nodal_solve(C, rh.data(), phi.data(), st);
    for (size_t c = 0; c < nc; ++c) {
        const double b = beta0 ? beta0[c] : 1.0;
        for (int d = 0; d < dm; ++d) unew[d * nc + c] /= b;
        rhoh[c] *= b;
        if (alt) rhoh[c] *= b;
    }
    std::vector<double> g(dm * nc);
    nodal_grad(C, F, phi.data(), g.data());
    // hg_update
    for (size_t c = 0; c < nc; ++c)
        for (int d = 0; d < dm; ++d) {
            double gv = g[d * nc + c];
            if (alt) gv *= (beta0 ? beta0[c] : 1.0);
            g[d * nc + c] = gv;
            double& u = unew[d * nc + c];
            u -= gv / rhoh[c];
            if (o->proj_type == HG_PRESSURE_ITERS) u = uold[d * nc + c] + o->dt * u;
        }
    if (o->proj_type == HG_INITIAL || o->proj_type == HG_DIVU_ITERS) {
        std::fill(gpi, gpi + dm * nc, 0.0);
        std::fill(pi, pi + nn, 0.0);
    } else if (o->proj_type == HG_PRESSURE_ITERS) {
        for (size_t q = 0; q < dm * nc; ++q) gpi[q] += g[q];
        for (size_t q = 0; q < nn; ++q) pi[q] += phi[q];
    } else if (o->proj_type == HG_REGULAR) {
        for (size_t q = 0; q < dm * nc; ++q) gpi[q] = g[q] / o->dt;
        for (size_t q = 0; q < nn; ++q) pi[q] = phi[q] / o->dt;
    }
    if (phi_out) std::copy(phi.begin(), phi.end(), phi_out);
    return status;
}

}  // extern "C"
