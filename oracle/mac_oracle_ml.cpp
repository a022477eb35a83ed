// Multi-level (AMR) MAC-projection oracle: a CPU (C++17 + OpenMP, IEEE FP64) restatement of
// MAESTRO's `macproject` on nlevs > 1 and of the FBoxLib composite (multi-level) cell-centred
// solve `ml_cc_solve` that `mac_multigrid` calls.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product path may link, load or call it.
//
// What it follows (paths are within the MAESTRO source tree):
//   Source/macproject.f90:154-161     beta0 U on every level
//   Source/macproject.f90:356-361     divumac: fine faces averaged onto the coarse faces they tile
//                                     (ml_edge_restriction) before the divergence
//   Source/macproject.f90:399-406     rh = -(div(beta0 U) - macrhs) on every level, then the
//                                     coarse rh under a finer level = mean of the fine rh
//                                     (ml_cc_restriction), finest first
//   Source/macproject.f90:182-203     solver_beta = beta0^p / rho_face on every level
//   Source/macproject.f90:217         rel_solver_eps = min(eps_mac * mac_level_factor^(nlevs-1),
//                                     eps_mac_max) (the caller passes it in o->rel_eps)
//   Source/macproject.f90:793-833     mkumac on every level with the solver's fluxes on box faces
//                                     (fine_flx), then ml_edge_restriction, finest first
//   Source/macproject.f90:230-265     divide out beta0, then ml_edge_restriction again
//   Docs/mg/mg.tex:124-155            bndry_reg: coarse data interpolated to the fine boundary;
//                                     the coarse residual next to a fine grid takes the fine
//                                     face fluxes instead of the coarse one
//
// FBoxLib is not part of the MAESTRO tree.  The composite discretisation and the multi-level
// cycle below are written from its published description and the mathematics; the choices:
//   * data      : every AMR level is a dense array over its whole level domain (n0 * 2^l cells)
//                 with a mask of the cells its boxes cover.  Level 0 covers the domain.  Valid
//                 cells of level l = its region minus the region of level l+1 coarsened.
//   * nesting   : every level-l box is aligned to the ratio 2 (even lo, odd hi) and its coarsened
//                 cells, grown by one cell in every direction (diagonals included, periodic wrap,
//                 clipped at other domain faces), lie in the level-(l-1) region.
//   * C-F ghost : a fine cell next to the coarse-fine interface sees the ghost
//                     phi_g = phi_own / 3 + 2/3 * phi_c,
//                 the line through the first fine cell and the coarse value located at the
//                 centre of the coarse cell across the face (stencil_order = 2: the boundary
//                 value half a coarse cell from the face, one interior point).  phi_c is the
//                 coarse cell value corrected along each tangential direction at the ghost's
//                 offset +-1/4 by the quadratic through the coarse cell and its two tangential
//                 neighbours (one-sided linear where a neighbour lies outside a non-periodic
//                 domain face); no cross term.
//   * reflux    : a valid coarse cell next to a covered one takes, for that face, the mean of
//                 the fine fluxes through the 2^(dm-1) fine faces tiling it instead of the coarse
//                 flux (conservative composite operator).  Covered coarse values are the mean of
//                 their children (phi restricted after every cycle).
//   * cycle     : multiplicative multi-level V-cycle in correction form.  Down: on each AMR
//                 level l >= 1, nu1 GS-RB sweeps on the correction with homogeneous C-F ghosts,
//                 the level's defect, the covered coarse defect = mean of the fine defect and
//                 the reflux of the fine correction into the adjacent coarse defect.  Level 0:
//                 one V-cycle of the one-level multigrid (mac_oracle.cpp) on the whole domain.
//                 Up: the coarse correction interpolated (cell-centred multilinear, 3/4-1/4)
//                 into the level, the level's defect with the coarse correction as C-F data,
//                 nu2 GS-RB sweeps with homogeneous C-F ghosts, corrections summed.  Then
//                 phi += correction on every level and phi restricted onto covered cells.
//   * singular  : no Dirichlet face -> the volume-weighted mean of rh over all valid cells is
//                 removed, the mean of the level-0 defect before each level-0 V-cycle and the
//                 mean of the level-0 correction after it.
//   * converged : max over levels of ||composite residual||_inf on valid cells
//                 <= rel_eps * max over levels of ||rh||_inf on valid cells (or <= abs_eps).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mac_oracle_core.h"

namespace {

using namespace orc;

constexpr int kMaxAmrLevels = 8;

struct AmrLevel {
    int n[3];
    double h[3];
    std::vector<uint8_t> in;    // cell inside the level's boxes
    std::vector<uint8_t> cov;   // cell covered by the next finer level
    std::vector<double> b[3];   // face coefficients, natural face layout of the level domain
    std::vector<double> f, phi, res, uu, hold, tmp, du;
    size_t ncell() const { return (size_t)n[0] * n[1] * n[2]; }
    bool valid(size_t c) const { return in[c] && !cov[c]; }
};

struct Amr {
    orc_opts o;
    int dm = 0;
    int act[3] = {0, 0, 0};
    std::vector<AmrLevel> L;
    Ctx base;               // one-level MG hierarchy of level 0 (coarse correction)
    bool singular = false;
};

// Neighbour index along d of level l (periodic wrap); -1 outside a non-periodic domain face.
inline int nbr(const Amr& A, int l, int d, int q) {
    const int n = A.L[l].n[d];
    if (q < 0) return A.o.bc_lo[d] == ORC_BC_PER ? q + n : -1;
    if (q >= n) return A.o.bc_hi[d] == ORC_BC_PER ? q - n : -1;
    return q;
}

// Validate alignment and proper nesting and build the masks.  Returns false on a bad layout.
bool build_layout(Amr& A, int nlev, const int* nboxes, const int* boxes) {
    if (nlev < 1 || nlev > kMaxAmrLevels) return false;
    A.dm = A.o.dm;
    for (int d = 0; d < 3; ++d) A.act[d] = d < A.dm;
    A.L.assign(nlev, AmrLevel());
    for (int l = 0; l < nlev; ++l) {
        AmrLevel& V = A.L[l];
        for (int d = 0; d < 3; ++d) {
            V.n[d] = A.act[d] ? (A.o.n[d] << l) : 1;
            V.h[d] = A.act[d] ? A.o.dx[d] / (double)(1 << l) : A.o.dx[d];
        }
        V.in.assign(V.ncell(), l == 0 ? 1 : 0);
        V.cov.assign(V.ncell(), 0);
    }
    const int* bx = boxes;
    for (int l = 1; l < nlev; ++l) {
        AmrLevel& V = A.L[l];
        if (nboxes[l] < 1) return false;
        for (int b = 0; b < nboxes[l]; ++b, bx += 6) {
            const int* lo = bx;
            const int* hi = bx + 3;
            for (int d = 0; d < 3; ++d) {
                if (!A.act[d]) {
                    if (lo[d] != 0 || hi[d] != 0) return false;
                    continue;
                }
                if (lo[d] < 0 || hi[d] >= V.n[d] || hi[d] < lo[d]) return false;
                if ((lo[d] & 1) || !(hi[d] & 1)) return false;
            }
            for (int k = lo[2]; k <= hi[2]; ++k)
                for (int j = lo[1]; j <= hi[1]; ++j)
                    for (int i = lo[0]; i <= hi[0]; ++i) V.in[cidx(V.n, i, j, k)] = 1;
        }
    }
    // covered masks and the nesting check
    for (int l = 1; l < nlev; ++l) {
        const AmrLevel& F = A.L[l];
        AmrLevel& K = A.L[l - 1];
        for (int k = 0; k < F.n[2]; ++k)
            for (int j = 0; j < F.n[1]; ++j)
                for (int i = 0; i < F.n[0]; ++i) {
                    if (!F.in[cidx(F.n, i, j, k)]) continue;
                    const int c[3] = {i >> A.act[0], j >> A.act[1], k >> A.act[2]};
                    K.cov[cidx(K.n, c[0], c[1], c[2])] = 1;
                    for (int a2 = -A.act[2]; a2 <= A.act[2]; ++a2)
                        for (int a1 = -A.act[1]; a1 <= A.act[1]; ++a1)
                            for (int a0 = -A.act[0]; a0 <= A.act[0]; ++a0) {
                                const int q0 = nbr(A, l - 1, 0, c[0] + a0);
                                const int q1 = nbr(A, l - 1, 1, c[1] + a1);
                                const int q2 = nbr(A, l - 1, 2, c[2] + a2);
                                if (q0 < 0 || q1 < 0 || q2 < 0) continue;
                                if (!K.in[cidx(K.n, q0, q1, q2)]) return false;
                            }
                }
    }
    for (AmrLevel& V : A.L) {
        const size_t N = V.ncell();
        V.f.assign(N, 0.0);
        V.phi.assign(N, 0.0);
        V.res.assign(N, 0.0);
        V.uu.assign(N, 0.0);
        V.hold.assign(N, 0.0);
        V.tmp.assign(N, 0.0);
        V.du.assign(N, 0.0);
    }
    return true;
}

// Coarse value at the fine ghost cell q (level l, inside the domain, outside the level region)
// seen across a face normal to d: the level-(l-1) cell containing q, corrected along each
// tangential direction by the quadratic through its tangential neighbours at offset +-1/4.
double coarse_at_ghost(const Amr& A, int l, const int q[3], int d, const double* cu) {
    const AmrLevel& K = A.L[l - 1];
    const int c[3] = {q[0] >> A.act[0], q[1] >> A.act[1], q[2] >> A.act[2]};
    const double v0 = cu[cidx(K.n, c[0], c[1], c[2])];
    double v = v0;
    for (int t = 0; t < 3; ++t) {
        if (t == d || !A.act[t]) continue;
        const double del = (q[t] & 1) ? 0.25 : -0.25;
        int m[3] = {c[0], c[1], c[2]}, p[3] = {c[0], c[1], c[2]};
        m[t] = nbr(A, l - 1, t, c[t] - 1);
        p[t] = nbr(A, l - 1, t, c[t] + 1);
        const bool hm = m[t] >= 0, hp = p[t] >= 0;
        const double vm = hm ? cu[cidx(K.n, m[0], m[1], m[2])] : 0.0;
        const double vp = hp ? cu[cidx(K.n, p[0], p[1], p[2])] : 0.0;
        if (hm && hp)
            v += del * 0.5 * (vp - vm) + 0.5 * del * del * (vp - 2.0 * v0 + vm);
        else if (hp)
            v += del * (vp - v0);
        else if (hm)
            v += del * (v0 - vm);
    }
    return v;
}

// Arm kinds of a level cell.
enum { ARM_IN = 0, ARM_NEU = 1, ARM_DIR = 2, ARM_CF = 3 };

inline int arm_kind(const Amr& A, int l, const int c[3], int d, int s, int q[3]) {
    q[0] = c[0];
    q[1] = c[1];
    q[2] = c[2];
    const int w = nbr(A, l, d, c[d] + s);
    if (w < 0) {
        const int bc = s < 0 ? A.o.bc_lo[d] : A.o.bc_hi[d];
        return bc == ORC_BC_DIR ? ARM_DIR : ARM_NEU;
    }
    q[d] = w;
    return A.L[l].in[cidx(A.L[l].n, q[0], q[1], q[2])] ? ARM_IN : ARM_CF;
}

inline double face_b(const AmrLevel& V, int d, const int c[3], int s) {
    int f[3] = {c[0], c[1], c[2]};
    if (s > 0) f[d] += 1;
    return V.b[d][fidx(V.n, d, f[0], f[1], f[2])];
}

// (L u)_c on level l: sum over arms beta/h^2 (u_c - u_nb), C-F ghosts from cu (null: zero
// coarse data).  Also returns the diagonal and the off-diagonal part for Gauss-Seidel.
inline void cell_op(const Amr& A, int l, const int c[3], const double* u, const double* cu,
                    double& diag, double& off) {
    const AmrLevel& V = A.L[l];
    diag = 0.0;
    off = 0.0;
    for (int d = 0; d < 3; ++d) {
        if (!A.act[d]) continue;
        const double ih2 = 1.0 / (V.h[d] * V.h[d]);
        for (int s = -1; s <= 1; s += 2) {
            int q[3];
            const int kind = arm_kind(A, l, c, d, s, q);
            const double w = face_b(V, d, c, s) * ih2;
            if (kind == ARM_IN) {
                diag += w;
                off += w * u[cidx(V.n, q[0], q[1], q[2])];
            } else if (kind == ARM_DIR) {
                diag += 2.0 * w;
            } else if (kind == ARM_CF) {
                diag += (2.0 / 3.0) * w;
                if (cu) off += (2.0 / 3.0) * w * coarse_at_ghost(A, l, q, d, cu);
            }
        }
    }
}

// r = f - L u on the region cells of level l (zero elsewhere); returns nothing.
void level_defect(const Amr& A, int l, const double* u, const double* cu, const double* f,
                  double* r) {
    const AmrLevel& V = A.L[l];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < V.n[2]; ++k)
        for (int j = 0; j < V.n[1]; ++j)
            for (int i = 0; i < V.n[0]; ++i) {
                const size_t c = cidx(V.n, i, j, k);
                if (!V.in[c]) {
                    r[c] = 0.0;
                    continue;
                }
                const int cc[3] = {i, j, k};
                double dg, off;
                cell_op(A, l, cc, u, cu, dg, off);
                r[c] = f[c] - (dg * u[c] - off);
            }
}

// nu red/black Gauss-Seidel sweeps of L u = f on the region of level l, homogeneous C-F ghosts.
void level_gsrb(const Amr& A, int l, double* u, const double* f, int nu) {
    const AmrLevel& V = A.L[l];
    for (int it = 0; it < nu; ++it)
        for (int colour = 0; colour < 2; ++colour) {
#pragma omp parallel for schedule(static)
            for (int k = 0; k < V.n[2]; ++k)
                for (int j = 0; j < V.n[1]; ++j)
                    for (int i = (j + k + colour) & 1; i < V.n[0]; i += 2) {
                        const size_t c = cidx(V.n, i, j, k);
                        if (!V.in[c]) continue;
                        const int cc[3] = {i, j, k};
                        double dg, off;
                        cell_op(A, l, cc, u, nullptr, dg, off);
                        u[c] = (f[c] + off) / dg;
                    }
        }
}

// For every valid level-(l-1) cell next to a cell covered by level l, replace the coarse arm
// through that face by the mean of the fine fluxes: res += (T_coarse - T_fine) / h.  uc = null
// means zero coarse data (T_coarse = 0 and coarse ghost data 0).
void cf_reflux(const Amr& A, int l, const double* uf, const double* uc, double* res) {
    const AmrLevel& K = A.L[l - 1];
    const AmrLevel& F = A.L[l];
    int ntan = 1;
    for (int d = 0; d < A.dm; ++d) ntan *= 2;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K.n[2]; ++k)
        for (int j = 0; j < K.n[1]; ++j)
            for (int i = 0; i < K.n[0]; ++i) {
                const size_t kc = cidx(K.n, i, j, k);
                if (!K.valid(kc)) continue;
                const int c[3] = {i, j, k};
                double acc = 0.0;
                for (int d = 0; d < 3; ++d) {
                    if (!A.act[d]) continue;
                    for (int s = -1; s <= 1; s += 2) {
                        int Q[3] = {i, j, k};
                        const int w = nbr(A, l - 1, d, c[d] + s);
                        if (w < 0) continue;
                        Q[d] = w;
                        if (!K.cov[cidx(K.n, Q[0], Q[1], Q[2])]) continue;
                        const double Tc = uc ? face_b(K, d, c, s) *
                                                   (uc[kc] - uc[cidx(K.n, Q[0], Q[1], Q[2])]) / K.h[d]
                                             : 0.0;
                        double Tf = 0.0;
                        const int nf = ntan / 2;
                        for (int a = 0; a < ntan; ++a) {
                            // tangential child offsets: bits of a over the active directions != d
                            int fc[3], gq[3];
                            bool skip = false;
                            for (int e = 0; e < 3; ++e) {
                                if (!A.act[e]) {
                                    fc[e] = gq[e] = 0;
                                    continue;
                                }
                                if (e == d) {
                                    fc[e] = s > 0 ? 2 * Q[e] : 2 * Q[e] + 1;
                                    gq[e] = s > 0 ? 2 * c[e] + 1 : 2 * c[e];
                                    if ((a >> e) & 1) skip = true;  // only a's with bit d clear
                                } else {
                                    fc[e] = gq[e] = 2 * c[e] + ((a >> e) & 1);
                                }
                            }
                            if (skip) continue;
                            const double ufv = uf[cidx(F.n, fc[0], fc[1], fc[2])];
                            const double g = ufv / 3.0 +
                                             (uc ? (2.0 / 3.0) * coarse_at_ghost(A, l, gq, d, uc) : 0.0);
                            // the fine cell's own arm towards the ghost (side -s)
                            const double bf = face_b(F, d, fc, -s);
                            Tf += bf * (g - ufv) / F.h[d];
                        }
                        Tf /= (double)nf;
                        acc += (Tc - Tf) / K.h[d];
                    }
                }
                res[kc] += acc;
            }
}

// Covered level-(l-1) cells take the mean of their 2^dm children of level l.
void restrict_covered(const Amr& A, int l, const double* fine, double* crse) {
    const AmrLevel& K = A.L[l - 1];
    const AmrLevel& F = A.L[l];
    const int r[3] = {A.act[0] ? 2 : 1, A.act[1] ? 2 : 1, A.act[2] ? 2 : 1};
    const double w = 1.0 / (r[0] * r[1] * r[2]);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K.n[2]; ++k)
        for (int j = 0; j < K.n[1]; ++j)
            for (int i = 0; i < K.n[0]; ++i) {
                const size_t kc = cidx(K.n, i, j, k);
                if (!K.cov[kc]) continue;
                double s = 0.0;
                for (int c2 = 0; c2 < r[2]; ++c2)
                    for (int c1 = 0; c1 < r[1]; ++c1)
                        for (int c0 = 0; c0 < r[0]; ++c0)
                            s += fine[cidx(F.n, i * r[0] + c0, j * r[1] + c1, k * r[2] + c2)];
                crse[kc] = s * w;
            }
}

// Max norm over the valid cells of every level of f (use_f) or of the residual.
double valid_norm(const Amr& A, bool use_f) {
    double mx = 0.0;
    bool nan = false;
    for (const AmrLevel& V : A.L) {
        const std::vector<double>& x = use_f ? V.f : V.res;
        for (size_t c = 0; c < V.ncell(); ++c)
            if (V.valid(c)) {
                nan = nan || std::isnan(x[c]);
                mx = std::max(mx, std::fabs(x[c]));
            }
    }
    return nan ? NAN : mx;
}

// Composite residual of phi on every level (valid cells; covered = mean of the fine residual).
// Returns its max norm over valid cells.
double composite_residual(Amr& A) {
    const int nl = (int)A.L.size();
    for (int l = 0; l < nl; ++l)
        level_defect(A, l, A.L[l].phi.data(), l ? A.L[l - 1].phi.data() : nullptr,
                     A.L[l].f.data(), A.L[l].res.data());
    for (int l = nl - 1; l >= 1; --l) {
        cf_reflux(A, l, A.L[l].phi.data(), A.L[l - 1].phi.data(), A.L[l - 1].res.data());
        restrict_covered(A, l, A.L[l].res.data(), A.L[l - 1].res.data());
    }
    return valid_norm(A, false);
}

// uf += multilinear interpolation of uc (level l-1) on the region cells of level l.
void prolong_region(const Amr& A, int l, const double* uc, double* uf) {
    const AmrLevel& K = A.L[l - 1];
    const AmrLevel& F = A.L[l];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < F.n[2]; ++k)
        for (int j = 0; j < F.n[1]; ++j)
            for (int i = 0; i < F.n[0]; ++i) {
                const size_t fcix = cidx(F.n, i, j, k);
                if (!F.in[fcix]) continue;
                const int fi[3] = {i, j, k};
                int pc[3], off[3];
                for (int d = 0; d < 3; ++d) {
                    pc[d] = A.act[d] ? fi[d] >> 1 : fi[d];
                    off[d] = A.act[d] ? ((fi[d] & 1) ? 1 : -1) : 0;
                }
                double s = 0.0;
                for (int a2 = 0; a2 < (off[2] ? 2 : 1); ++a2)
                    for (int a1 = 0; a1 < (off[1] ? 2 : 1); ++a1)
                        for (int a0 = 0; a0 < (off[0] ? 2 : 1); ++a0) {
                            const int a[3] = {a0, a1, a2};
                            double w = 1.0, sgn = 1.0;
                            int q[3];
                            for (int d = 0; d < 3; ++d) {
                                if (!off[d]) {
                                    q[d] = pc[d];
                                    continue;
                                }
                                w *= a[d] ? 0.25 : 0.75;
                                const int want = pc[d] + (a[d] ? off[d] : 0);
                                const int got = nbr(A, l - 1, d, want);
                                if (got >= 0) {
                                    q[d] = got;
                                } else {  // reflection at a physical face
                                    q[d] = pc[d];
                                    const int bc = want < 0 ? A.o.bc_lo[d] : A.o.bc_hi[d];
                                    if (bc == ORC_BC_DIR) sgn = -sgn;
                                }
                            }
                            s += w * sgn * uc[cidx(K.n, q[0], q[1], q[2])];
                        }
                uf[fcix] += s;
            }
}


void remove_composite_mean(Amr& A) {
    double s = 0.0, vol = 0.0;
    for (const AmrLevel& V : A.L) {
        const double cv = V.h[0] * V.h[1] * V.h[2];
        for (size_t c = 0; c < V.ncell(); ++c)
            if (V.valid(c)) {
                s += V.f[c] * cv;
                vol += cv;
            }
    }
    const double m = s / vol;
    for (AmrLevel& V : A.L)
        for (size_t c = 0; c < V.ncell(); ++c)
            if (V.valid(c)) V.f[c] -= m;
}

// One multi-level V-cycle on the current composite residual; adds the correction to phi.
void ml_vcycle(Amr& A) {
    const int nl = (int)A.L.size();
    const orc_opts& o = A.o;
    for (int l = nl - 1; l >= 1; --l) {
        AmrLevel& V = A.L[l];
        std::fill(V.uu.begin(), V.uu.end(), 0.0);
        level_gsrb(A, l, V.uu.data(), V.res.data(), o.nu1);
        level_defect(A, l, V.uu.data(), nullptr, V.res.data(), V.tmp.data());
        V.res.swap(V.tmp);
        V.hold = V.uu;
        restrict_covered(A, l, V.res.data(), A.L[l - 1].res.data());
        cf_reflux(A, l, V.uu.data(), nullptr, A.L[l - 1].res.data());
    }
    {
        Level& B = A.base.lev[0];
        B.f = A.L[0].res;
        if (A.singular) sub_mean(B.f);
        B.phi.assign(B.f.size(), 0.0);
        vcycle(A.base, 0);
        // the constant is in the null space of the composite operator: keep it out of the
        // correction (a drifting bottom solve would otherwise swamp phi's FP64 precision)
        if (A.singular) sub_mean(B.phi);
        A.L[0].uu = B.phi;
    }
    for (int l = 1; l < nl; ++l) {
        AmrLevel& V = A.L[l];
        std::fill(V.uu.begin(), V.uu.end(), 0.0);
        prolong_region(A, l, A.L[l - 1].uu.data(), V.uu.data());
        level_defect(A, l, V.uu.data(), A.L[l - 1].uu.data(), V.res.data(), V.tmp.data());
        std::fill(V.du.begin(), V.du.end(), 0.0);
        level_gsrb(A, l, V.du.data(), V.tmp.data(), o.nu2);
        for (size_t c = 0; c < V.ncell(); ++c)
            if (V.in[c]) V.uu[c] += V.hold[c] + V.du[c];
    }
    for (int l = 0; l < nl; ++l) {
        AmrLevel& V = A.L[l];
        for (size_t c = 0; c < V.ncell(); ++c)
            if (V.in[c]) V.phi[c] += V.uu[c];
    }
    for (int l = nl - 1; l >= 1; --l) restrict_covered(A, l, A.L[l].phi.data(), A.L[l - 1].phi.data());
}

bool has_dirichlet(const orc_opts& o) {
    for (int d = 0; d < o.dm; ++d)
        if (o.bc_lo[d] == ORC_BC_DIR || o.bc_hi[d] == ORC_BC_DIR) return true;
    return false;
}

// Face coefficients of every level copied in (natural face layout of each level domain).
void load_beta(Amr& A, const double* const* beta) {
    for (size_t l = 0; l < A.L.size(); ++l) {
        AmrLevel& V = A.L[l];
        for (int d = 0; d < 3; ++d) {
            if (!A.act[d]) continue;
            const size_t m = (size_t)(V.n[0] + (d == 0)) * (V.n[1] + (d == 1)) * (V.n[2] + (d == 2));
            const double* p = beta[3 * l + d];
            V.b[d].assign(p, p + m);
        }
    }
    const double* b0[3] = {A.L[0].b[0].data(), A.L[0].b[1].data(),
                           A.act[2] ? A.L[0].b[2].data() : nullptr};
    A.base = Ctx();
    A.base.o = A.o;
    build_hierarchy(A.base, b0, nullptr);
    A.singular = !has_dirichlet(A.o);
}

int ml_solve(Amr& A, const double* const* rh, double* const* phi, orc_stats* st) {
    const int nl = (int)A.L.size();
    for (int l = 0; l < nl; ++l) {
        AmrLevel& V = A.L[l];
        V.f.assign(rh[l], rh[l] + V.ncell());
        V.phi.assign(phi[l], phi[l] + V.ncell());
        for (size_t c = 0; c < V.ncell(); ++c)
            if (!V.in[c]) V.phi[c] = 0.0;
    }
    if (A.singular) remove_composite_mean(A);
    for (int l = nl - 1; l >= 1; --l) restrict_covered(A, l, A.L[l].phi.data(), A.L[l - 1].phi.data());
    orc_stats local{};
    orc_stats& S = st ? *st : local;
    std::memset(&S, 0, sizeof(S));
    const double fnorm = valid_norm(A, true);
    S.fnorm = fnorm;
    auto out = [&]() {
        for (int l = 0; l < nl; ++l) std::copy(A.L[l].phi.begin(), A.L[l].phi.end(), phi[l]);
    };
    if (fnorm == 0.0) {
        for (AmrLevel& V : A.L) std::fill(V.phi.begin(), V.phi.end(), 0.0);
        out();
        return 0;
    }
    auto converged = [&](double r) {
        return r <= A.o.rel_eps * fnorm || (A.o.abs_eps > 0.0 && r <= A.o.abs_eps);
    };
    double res = composite_residual(A);
    S.resid0 = res;
    int it = 0;
    while (!converged(res) && it < A.o.max_vcycles) {
        ml_vcycle(A);
        ++it;
        res = composite_residual(A);
        if (S.nhist < 64) S.hist[S.nhist++] = res / fnorm;
    }
    S.vcycles = it;
    S.rel_resid = res / fnorm;
    S.status = converged(res) ? 0 : 1;
    S.bottom_iters = A.base.bottom_iters;
    out();
    return S.status;
}

// A fine face (d, f) of level l belongs to the level when a cell on either side is in it.
inline bool face_in_level(const Amr& A, int l, int d, const int f[3]) {
    const AmrLevel& V = A.L[l];
    int hi[3] = {f[0], f[1], f[2]}, lo[3] = {f[0], f[1], f[2]};
    lo[d] = nbr(A, l, d, f[d] - 1);
    hi[d] = f[d] < V.n[d] ? f[d] : nbr(A, l, d, f[d]);
    return (lo[d] >= 0 && V.in[cidx(V.n, lo[0], lo[1], lo[2])]) ||
           (hi[d] >= 0 && V.in[cidx(V.n, hi[0], hi[1], hi[2])]);
}

// ml_edge_restriction: every level-(l-1) face tiled by level-l faces takes their mean.
void edge_restrict(const Amr& A, int l, double* const* uc, double* const* uf) {
    const AmrLevel& K = A.L[l - 1];
    const AmrLevel& F = A.L[l];
    for (int d = 0; d < 3; ++d) {
        if (!A.act[d]) continue;
        const int m[3] = {K.n[0] + (d == 0), K.n[1] + (d == 1), K.n[2] + (d == 2)};
        int ntan = 1;
        for (int e = 0; e < 3; ++e)
            if (e != d && A.act[e]) ntan *= 2;
#pragma omp parallel for schedule(static)
        for (int k = 0; k < m[2]; ++k)
            for (int j = 0; j < m[1]; ++j)
                for (int i = 0; i < m[0]; ++i) {
                    const int cf[3] = {i, j, k};
                    int f0[3];
                    for (int e = 0; e < 3; ++e) f0[e] = A.act[e] ? 2 * cf[e] : cf[e];
                    if (!face_in_level(A, l, d, f0)) continue;
                    double s = 0.0;
                    for (int a = 0; a < 8; ++a) {
                        int f[3] = {f0[0], f0[1], f0[2]};
                        bool skip = false;
                        for (int e = 0; e < 3; ++e) {
                            const int bit = (a >> e) & 1;
                            if (e == d || !A.act[e]) {
                                if (bit) skip = true;
                            } else {
                                f[e] += bit;
                            }
                        }
                        if (skip) continue;
                        s += uf[d][fidx(F.n, d, f[0], f[1], f[2])];
                    }
                    uc[d][fidx(K.n, d, i, j, k)] = s / ntan;
                }
    }
}

// mkumac on level l: beta0 U -= beta_f * G phi on every face of the level; C-F faces use the
// ghost of the composite operator (coarse phi of level l-1); other faces as on one level.
void correct_level(const Amr& A, int l, double* const* u) {
    const AmrLevel& V = A.L[l];
    const double* phi = V.phi.data();
    const double* cu = l ? A.L[l - 1].phi.data() : nullptr;
    for (int d = 0; d < 3; ++d) {
        if (!A.act[d]) continue;
        const int m[3] = {V.n[0] + (d == 0), V.n[1] + (d == 1), V.n[2] + (d == 2)};
#pragma omp parallel for schedule(static)
        for (int k = 0; k < m[2]; ++k)
            for (int j = 0; j < m[1]; ++j)
                for (int i = 0; i < m[0]; ++i) {
                    const int f[3] = {i, j, k};
                    if (!face_in_level(A, l, d, f)) continue;
                    int lo[3] = {i, j, k}, hi[3] = {i, j, k};
                    lo[d] = nbr(A, l, d, f[d] - 1);
                    hi[d] = f[d] < V.n[d] ? f[d] : nbr(A, l, d, f[d]);
                    const bool lin = lo[d] >= 0 && V.in[cidx(V.n, lo[0], lo[1], lo[2])];
                    const bool hin = hi[d] >= 0 && V.in[cidx(V.n, hi[0], hi[1], hi[2])];
                    double g;
                    if (lin && hin) {
                        g = (phi[cidx(V.n, hi[0], hi[1], hi[2])] - phi[cidx(V.n, lo[0], lo[1], lo[2])]) / V.h[d];
                    } else if (hin && lo[d] < 0) {
                        g = (A.o.bc_lo[d] == ORC_BC_DIR) ? 2.0 * phi[cidx(V.n, hi[0], hi[1], hi[2])] / V.h[d] : 0.0;
                    } else if (lin && hi[d] < 0) {
                        g = (A.o.bc_hi[d] == ORC_BC_DIR) ? -2.0 * phi[cidx(V.n, lo[0], lo[1], lo[2])] / V.h[d] : 0.0;
                    } else if (hin) {  // C-F face on the low side of the region
                        const double pv = phi[cidx(V.n, hi[0], hi[1], hi[2])];
                        const double gv = pv / 3.0 + (2.0 / 3.0) * coarse_at_ghost(A, l, lo, d, cu);
                        g = (pv - gv) / V.h[d];
                    } else {           // C-F face on the high side of the region
                        const double pv = phi[cidx(V.n, lo[0], lo[1], lo[2])];
                        const double gv = pv / 3.0 + (2.0 / 3.0) * coarse_at_ghost(A, l, hi, d, cu);
                        g = (gv - pv) / V.h[d];
                    }
                    const size_t fi = fidx(V.n, d, i, j, k);
                    u[d][fi] -= V.b[d][fi] * g;
                }
    }
}

orc_opts level_opts(const Amr& A, int l) {
    orc_opts o = A.o;
    for (int d = 0; d < 3; ++d) {
        o.n[d] = A.L[l].n[d];
        o.dx[d] = A.L[l].h[d];
    }
    return o;
}

}  // namespace

extern "C" {

// Composite solve of -div(beta grad phi) = rh over nlev AMR levels.  Level l arrays span the
// whole level domain (n[d] << l cells along the active directions; Fortran order); rh[l],
// phi[l] cells; beta[3 l + d] faces (n_l[d] + 1 along d).  nboxes[l] boxes for l >= 1 follow
// in `boxes` as lo[3], hi[3] in level-l indices (nboxes[0] is ignored).  phi is the initial
// guess on entry and holds the solution on exit, covered cells = mean of their children.
// Returns 0 converged, 1 not converged, -1 an invalid layout (alignment or nesting).
int orc_ml_solve(const orc_opts* o, int nlev, const int* nboxes, const int* boxes,
                 const double* const* rh, double* const* phi, const double* const* beta,
                 orc_stats* st) {
    set_threads(o);
    Amr A;
    A.o = *o;
    if (!build_layout(A, nlev, nboxes, boxes)) return -1;
    load_beta(A, beta);
    return ml_solve(A, rh, phi, st);
}

// Composite residual rh - L phi on every level (covered cells = mean of their children's
// residual, cells outside a level's region 0); returns its max over valid cells, or -1 on an
// invalid layout.  rh is used as given (no mean removal).
double orc_ml_residual(const orc_opts* o, int nlev, const int* nboxes, const int* boxes,
                       const double* const* rh, const double* const* phi,
                       const double* const* beta, double* const* res) {
    set_threads(o);
    Amr A;
    A.o = *o;
    A.o.nlevels = 1;
    if (!build_layout(A, nlev, nboxes, boxes)) return -1.0;
    load_beta(A, beta);
    for (int l = 0; l < nlev; ++l) {
        AmrLevel& V = A.L[l];
        V.f.assign(rh[l], rh[l] + V.ncell());
        V.phi.assign(phi[l], phi[l] + V.ncell());
    }
    const double r = composite_residual(A);
    for (int l = 0; l < nlev; ++l)
        if (res && res[l]) std::copy(A.L[l].res.begin(), A.L[l].res.end(), res[l]);
    return r;
}

// Multi-level MAC projection (Source/macproject.f90:51-328 with nlevs > 1).  u[3 l + d] are the
// face velocities of level l (natural face layout of the level domain; only faces of the level's
// region are read or written), phi[l] the cell potential (in: initial guess), rho[l] the cell
// density on the level region plus one ghost layer, macrhs[l] (macrhs null or an entry null:
// none) the cell source, beta0[l] / beta0_edge[l] (nullable together) the planar base state of
// level l (n_l[dm-1] and n_l[dm-1] + 1 entries).  Returns as orc_ml_solve.
int orc_macproject_ml(const orc_opts* o, int nlev, const int* nboxes, const int* boxes,
                      double* const* u, double* const* phi, const double* const* rho,
                      const double* const* macrhs, const double* const* beta0,
                      const double* const* beta0_edge, orc_stats* st) {
    set_threads(o);
    Amr A;
    A.o = *o;
    if (!build_layout(A, nlev, nboxes, boxes)) return -1;
    const int dm = A.dm;
    const int va = dm - 1;
    auto scale = [&](int l, bool mult) {
        if (!beta0) return;
        const AmrLevel& V = A.L[l];
        for (int d = 0; d < dm; ++d) {
            const int m[3] = {V.n[0] + (d == 0), V.n[1] + (d == 1), V.n[2] + (d == 2)};
            double* x = u[3 * l + d];
#pragma omp parallel for schedule(static)
            for (int k = 0; k < m[2]; ++k)
                for (int j = 0; j < m[1]; ++j)
                    for (int i = 0; i < m[0]; ++i) {
                        const int r = va == 0 ? i : va == 1 ? j : k;
                        const double bb = d == va ? beta0_edge[l][r] : beta0[l][r];
                        double& v = x[fidx(V.n, d, i, j, k)];
                        v = mult ? v * bb : v / bb;
                    }
        }
    };
    for (int l = 0; l < nlev; ++l) scale(l, true);
    for (int l = nlev - 1; l >= 1; --l) edge_restrict(A, l, u + 3 * (l - 1), u + 3 * l);

    // divumac on every level, then the coarse rh under a finer level = mean of the fine rh
    std::vector<std::vector<double>> rh(nlev);
    for (int l = 0; l < nlev; ++l) {
        const AmrLevel& V = A.L[l];
        rh[l].assign(V.ncell(), 0.0);
        const double* mr = macrhs ? macrhs[l] : nullptr;
#pragma omp parallel for schedule(static)
        for (int k = 0; k < V.n[2]; ++k)
            for (int j = 0; j < V.n[1]; ++j)
                for (int i = 0; i < V.n[0]; ++i) {
                    const size_t c = cidx(V.n, i, j, k);
                    if (!V.in[c]) continue;
                    double dv = 0.0;
                    for (int d = 0; d < dm; ++d) {
                        int hi[3] = {i, j, k};
                        hi[d] += 1;
                        dv += (u[3 * l + d][fidx(V.n, d, hi[0], hi[1], hi[2])] -
                               u[3 * l + d][fidx(V.n, d, i, j, k)]) / V.h[d];
                    }
                    if (mr) dv -= mr[c];
                    rh[l][c] = -dv;
                }
    }
    for (int l = nlev - 1; l >= 1; --l) restrict_covered(A, l, rh[l].data(), rh[l - 1].data());

    // solver_beta = beta0^p * 2 / (rho_L + rho_R) on every level
    std::vector<std::vector<double>> bf(3 * nlev);
    std::vector<const double*> bp(3 * nlev, nullptr);
    for (int l = 0; l < nlev; ++l) {
        const AmrLevel& V = A.L[l];
        for (int d = 0; d < 3; ++d) {
            const size_t m = d < dm ? (size_t)(V.n[0] + (d == 0)) * (V.n[1] + (d == 1)) * (V.n[2] + (d == 2)) : 1;
            bf[3 * l + d].assign(m, 0.0);
            bp[3 * l + d] = bf[3 * l + d].data();
        }
        const orc_opts lo = level_opts(A, l);
        orc_mac_coeffs(&lo, rho[l], beta0 ? beta0[l] : nullptr, beta0 ? beta0_edge[l] : nullptr,
                       bf[3 * l].data(), bf[3 * l + 1].data(), bf[3 * l + 2].data());
    }
    load_beta(A, bp.data());

    std::vector<const double*> rp(nlev);
    for (int l = 0; l < nlev; ++l) rp[l] = rh[l].data();
    const int status = ml_solve(A, rp.data(), phi, st);

    // mkumac on every level, then ml_edge_restriction; divide out beta0; restrict again
    for (int l = 0; l < nlev; ++l) correct_level(A, l, u + 3 * l);
    for (int l = nlev - 1; l >= 1; --l) edge_restrict(A, l, u + 3 * (l - 1), u + 3 * l);
    for (int l = 0; l < nlev; ++l) scale(l, false);
    for (int l = nlev - 1; l >= 1; --l) edge_restrict(A, l, u + 3 * (l - 1), u + 3 * l);
    return status;
}

}  // extern "C"
