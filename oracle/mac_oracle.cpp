// MAC-projection oracle: a CPU (C++17 + OpenMP, IEEE FP64) restatement of MAESTRO's
// `macproject` and of the FBoxLib cell-centred geometric multigrid that `mac_multigrid`
// hands the elliptic solve to.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA library in
// maestro_gb300/csrc and the timed CPU baseline of bench.py.  Nothing in the product
// path may link, load or call it.
//
// What it follows (paths are within the MAESTRO source tree):
//   Source/macproject.f90:51-328     macproject driver (order of steps, signs)
//   Source/macproject.f90:482-609    mult_edge_by_1d_coeff: x/y faces * beta0(k), z faces * beta0_edge(k)
//   Source/macproject.f90:385-398    rh = -(div(beta0 U) - macrhs)
//   Source/macproject.f90:457-480    divumac_3d
//   Source/macproject.f90:698-738    mk_mac_coeffs_3d: beta_f = 2 / (rho_L + rho_R)
//   Source/macproject.f90:184-203    solver_beta *= beta0 (twice when use_alt_energy_fix)
//   Source/macproject.f90:908-975    mkumac_3d: beta0 U -= beta_f * (phi_i - phi_{i-1}) / dx
//   Source/mac_multigrid.f90:56-67   ml_cc_solve parameters: nub, V-cycle, bottom eps 1e-3
//   Source/mg_eps.f90:23-28          eps_mac = 1e-10, eps_mac_max = 1e-8, level factor 10
//   Source/cell_to_edge.f90:14-70    beta0 cell -> edge (limited 4th order)
//   Source/define_bc_tower.f90:329-392  press_comp elliptic BCs (slip wall -> Neumann, ...)
//   Docs/mg/mg.tex:196-259, 325-375  GS-RB smoother, V-cycle flow, conservative restriction,
//                                    linear prolongation for 2x jumps, BiCGStab bottom solve,
//                                    coarsening of every box down to 2 cells per side
//
// FBoxLib itself is not part of the MAESTRO tree (external, unpinned dependency), so the MG
// arithmetic below is written from its published description and the mathematics; the
// choices made where the description is silent are listed next to the code:
//   * operator   : (alpha - div beta grad) phi with the 7-point (3D) / 5-point (2D) cross stencil,
//                  face coefficients beta_f, Neumann faces dropped, periodic faces wrapped,
//                  homogeneous Dirichlet faces with the linear ghost phi_g = -phi_0
//                  (contributes 2 beta_f / h^2 to the diagonal).
//   * smoother   : red/black Gauss-Seidel, colour = (i+j+k) mod 2 in global indices, even cells first.
//   * coarsening : face coefficients of a coarse face = mean of the fine faces covering it;
//                  h doubles; defect restricted by the mean of the 2^dm children.
//   * prolongation: cell-centred (bi/tri)linear interpolation, weights 3/4, 1/4 per direction,
//                  coarse ghosts by periodic wrap / even (Neumann) / odd (Dirichlet) reflection.
//   * bottom     : nub GS-RB sweeps, Jacobi-preconditioned BiCGStab to bottom_eps (relative,
//                  max-norm) on the coarsest level, nub GS-RB sweeps.
//   * singular   : alpha == 0 and no Dirichlet face -> mean of the right-hand side removed on the
//                  finest level and before every bottom solve.
//   * convergence: ||f - L phi||_inf <= rel_eps * ||f||_inf  (or <= abs_eps when abs_eps > 0).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mac_oracle_core.h"

namespace orc {

void build_diag(Ctx& C, Level& L) {
    const orc_opts& o = C.o;
    const int* n = L.n;
    L.diag.assign(L.ncell(), 0.0);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n[2]; ++k)
        for (int j = 0; j < n[1]; ++j)
            for (int i = 0; i < n[0]; ++i) {
                const int c[3] = {i, j, k};
                double s = L.alpha.empty() ? 0.0 : L.alpha[cidx(n, i, j, k)];
                for (int d = 0; d < 3; ++d) {
                    if (!L.act[d]) continue;
                    const double ih2 = 1.0 / (L.h[d] * L.h[d]);
                    int lo[3] = {i, j, k}, hi[3] = {i, j, k};
                    hi[d] += 1;
                    const double blo = L.b[d][fidx(n, d, lo[0], lo[1], lo[2])];
                    const double bhi = L.b[d][fidx(n, d, hi[0], hi[1], hi[2])];
                    // low face
                    if (c[d] > 0 || o.bc_lo[d] == ORC_BC_PER) s += blo * ih2;
                    else if (o.bc_lo[d] == ORC_BC_DIR) s += 2.0 * blo * ih2;
                    // high face
                    if (c[d] < n[d] - 1 || o.bc_hi[d] == ORC_BC_PER) s += bhi * ih2;
                    else if (o.bc_hi[d] == ORC_BC_DIR) s += 2.0 * bhi * ih2;
                }
                L.diag[cidx(n, i, j, k)] = s;
            }
}

// Sum over the stencil arms of beta_f/h^2 * phi_neighbour (the off-diagonal part, sign +).
inline double offdiag_sum(const Ctx& C, const Level& L, const double* u, int i, int j, int k) {
    const orc_opts& o = C.o;
    const int* n = L.n;
    const int c[3] = {i, j, k};
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        if (!L.act[d]) continue;
        const double ih2 = 1.0 / (L.h[d] * L.h[d]);
        int lo[3] = {i, j, k}, hi[3] = {i, j, k};
        hi[d] += 1;
        const int ql = nb_index(c[d], -1, n[d], o.bc_lo[d], o.bc_hi[d]);
        const int qh = nb_index(c[d], +1, n[d], o.bc_lo[d], o.bc_hi[d]);
        if (ql >= 0) {
            int p[3] = {i, j, k};
            p[d] = ql;
            s += L.b[d][fidx(n, d, lo[0], lo[1], lo[2])] * ih2 * u[cidx(n, p[0], p[1], p[2])];
        }
        if (qh >= 0) {
            int p[3] = {i, j, k};
            p[d] = qh;
            s += L.b[d][fidx(n, d, hi[0], hi[1], hi[2])] * ih2 * u[cidx(n, p[0], p[1], p[2])];
        }
    }
    return s;
}

void apply_op(const Ctx& C, const Level& L, const double* u, double* out) {
    const int* n = L.n;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n[2]; ++k)
        for (int j = 0; j < n[1]; ++j)
            for (int i = 0; i < n[0]; ++i) {
                const size_t c = cidx(n, i, j, k);
                out[c] = L.diag[c] * u[c] - offdiag_sum(C, L, u, i, j, k);
            }
}

double residual(const Ctx& C, const Level& L, const double* u, const double* f, double* r) {
    const int* n = L.n;
    double mx = 0.0;
#pragma omp parallel for schedule(static) reduction(max : mx)
    for (int k = 0; k < n[2]; ++k)
        for (int j = 0; j < n[1]; ++j)
            for (int i = 0; i < n[0]; ++i) {
                const size_t c = cidx(n, i, j, k);
                const double v = f[c] - (L.diag[c] * u[c] - offdiag_sum(C, L, u, i, j, k));
                if (r) r[c] = v;
                mx = std::max(mx, std::fabs(v));
            }
    return mx;
}

// One red/black Gauss-Seidel sweep (even colour first), FBoxLib MG_SMOOTHER_GS_RB.
void gsrb(const Ctx& C, Level& L) {
    const int* n = L.n;
    for (int colour = 0; colour < 2; ++colour) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n[2]; ++k)
            for (int j = 0; j < n[1]; ++j)
                for (int i = (j + k + colour) & 1; i < n[0]; i += 2) {
                    const size_t c = cidx(n, i, j, k);
                    L.phi[c] = (L.f[c] + offdiag_sum(C, L, L.phi.data(), i, j, k)) / L.diag[c];
                }
    }
}

double mean_of(const std::vector<double>& v) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long q = 0; q < (long)v.size(); ++q) s += v[q];
    return s / (double)v.size();
}

void sub_mean(std::vector<double>& v) {
    const double m = mean_of(v);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)v.size(); ++q) v[q] -= m;
}

double norm_inf(const std::vector<double>& v) {
    double mx = 0.0;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (long q = 0; q < (long)v.size(); ++q) mx = std::max(mx, std::fabs(v[q]));
    return mx;
}

// Coarse level from a fine one: h doubles in the active directions, each coarse face takes the
// mean of the fine faces that tile it.
void coarsen_level(const Ctx& C, const Level& F, Level& K) {
    for (int d = 0; d < 3; ++d) {
        K.act[d] = F.act[d];
        const int r = F.act[d] ? 2 : 1;
        K.n[d] = F.n[d] / r;
        K.h[d] = F.h[d] * r;
    }
    const int r[3] = {F.act[0] ? 2 : 1, F.act[1] ? 2 : 1, F.act[2] ? 2 : 1};
    for (int d = 0; d < 3; ++d) {
        if (!K.act[d]) continue;
        const int m[3] = {K.n[0] + (d == 0), K.n[1] + (d == 1), K.n[2] + (d == 2)};
        K.b[d].assign((size_t)m[0] * m[1] * m[2], 0.0);
        int cnt = 1;
        for (int e = 0; e < 3; ++e)
            if (e != d) cnt *= r[e];
#pragma omp parallel for schedule(static)
        for (int k = 0; k < m[2]; ++k)
            for (int j = 0; j < m[1]; ++j)
                for (int i = 0; i < m[0]; ++i) {
                    const int base[3] = {i * r[0], j * r[1], k * r[2]};
                    double s = 0.0;
                    for (int c2 = 0; c2 < (d == 2 ? 1 : r[2]); ++c2)
                        for (int c1 = 0; c1 < (d == 1 ? 1 : r[1]); ++c1)
                            for (int c0 = 0; c0 < (d == 0 ? 1 : r[0]); ++c0)
                                s += F.b[d][fidx(F.n, d, base[0] + c0, base[1] + c1, base[2] + c2)];
                    K.b[d][fidx(K.n, d, i, j, k)] = s / cnt;
                }
    }
    if (!F.alpha.empty()) {
        K.alpha.assign(K.ncell(), 0.0);
        const double w = 1.0 / (r[0] * r[1] * r[2]);
        for (int k = 0; k < K.n[2]; ++k)
            for (int j = 0; j < K.n[1]; ++j)
                for (int i = 0; i < K.n[0]; ++i) {
                    double s = 0.0;
                    for (int c2 = 0; c2 < r[2]; ++c2)
                        for (int c1 = 0; c1 < r[1]; ++c1)
                            for (int c0 = 0; c0 < r[0]; ++c0)
                                s += F.alpha[cidx(F.n, i * r[0] + c0, j * r[1] + c1, k * r[2] + c2)];
                    K.alpha[cidx(K.n, i, j, k)] = s * w;
                }
    }
    K.phi.assign(K.ncell(), 0.0);
    K.f.assign(K.ncell(), 0.0);
    K.r.assign(K.ncell(), 0.0);
}

void restrict_defect(const Level& F, Level& K) {
    const int r[3] = {F.act[0] ? 2 : 1, F.act[1] ? 2 : 1, F.act[2] ? 2 : 1};
    const double w = 1.0 / (r[0] * r[1] * r[2]);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K.n[2]; ++k)
        for (int j = 0; j < K.n[1]; ++j)
            for (int i = 0; i < K.n[0]; ++i) {
                double s = 0.0;
                for (int c2 = 0; c2 < r[2]; ++c2)
                    for (int c1 = 0; c1 < r[1]; ++c1)
                        for (int c0 = 0; c0 < r[0]; ++c0)
                            s += F.r[cidx(F.n, i * r[0] + c0, j * r[1] + c1, k * r[2] + c2)];
                K.f[cidx(K.n, i, j, k)] = s * w;
            }
}

// Coarse value at (possibly out-of-range) index q along d, with the BC-dependent reflection.
inline double coarse_ghost_factor(int& q, int nd, int bclo, int bchi) {
    if (q < 0) {
        if (bclo == ORC_BC_PER) { q = nd - 1; return 1.0; }
        q = 0;
        return bclo == ORC_BC_DIR ? -1.0 : 1.0;
    }
    if (q >= nd) {
        if (bchi == ORC_BC_PER) { q = 0; return 1.0; }
        q = nd - 1;
        return bchi == ORC_BC_DIR ? -1.0 : 1.0;
    }
    return 1.0;
}

void prolong_add(const Ctx& C, const Level& K, Level& F) {
    const orc_opts& o = C.o;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < F.n[2]; ++k)
        for (int j = 0; j < F.n[1]; ++j)
            for (int i = 0; i < F.n[0]; ++i) {
                const int fi[3] = {i, j, k};
                int pc[3], off[3];
                for (int d = 0; d < 3; ++d) {
                    if (F.act[d]) {
                        pc[d] = fi[d] >> 1;
                        off[d] = (fi[d] & 1) ? 1 : -1;
                    } else {
                        pc[d] = fi[d];
                        off[d] = 0;
                    }
                }
                double s = 0.0;
                for (int a2 = 0; a2 < (off[2] ? 2 : 1); ++a2)
                    for (int a1 = 0; a1 < (off[1] ? 2 : 1); ++a1)
                        for (int a0 = 0; a0 < (off[0] ? 2 : 1); ++a0) {
                            const int a[3] = {a0, a1, a2};
                            double w = 1.0, sgn = 1.0;
                            int q[3];
                            for (int d = 0; d < 3; ++d) {
                                if (!off[d]) { q[d] = pc[d]; continue; }
                                w *= a[d] ? 0.25 : 0.75;
                                q[d] = pc[d] + (a[d] ? off[d] : 0);
                                sgn *= coarse_ghost_factor(q[d], K.n[d], o.bc_lo[d], o.bc_hi[d]);
                            }
                            s += w * sgn * K.phi[cidx(K.n, q[0], q[1], q[2])];
                        }
                F.phi[cidx(F.n, i, j, k)] += s;
            }
}

// Jacobi-preconditioned BiCGStab on the coarsest level; reduces ||f - L phi||_inf by bottom_eps.
void bottom_bicgstab(Ctx& C, Level& L) {
    const size_t N = L.ncell();
    std::vector<double> r(N), rh(N), p(N, 0.0), v(N, 0.0), ph(N), s(N), sh(N), t(N);
    std::vector<double>& x = L.phi;
    if (C.singular) sub_mean(L.f);
    residual(C, L, x.data(), L.f.data(), r.data());
    const double r0 = norm_inf(r);
    if (r0 == 0.0) return;
    const double tol = C.o.bottom_eps * r0;
    rh = r;
    double rho_old = 1.0, alpha = 1.0, omega = 1.0;
    auto dot = [&](const std::vector<double>& a, const std::vector<double>& b) {
        double acc = 0.0;
        for (size_t q = 0; q < N; ++q) acc += a[q] * b[q];
        return acc;
    };
    for (int it = 0; it < C.o.bottom_max_iter; ++it) {
        C.bottom_iters++;
        const double rho = dot(rh, r);
        if (rho == 0.0) break;
        const double beta = (rho / rho_old) * (alpha / omega);
        for (size_t q = 0; q < N; ++q) p[q] = r[q] + beta * (p[q] - omega * v[q]);
        for (size_t q = 0; q < N; ++q) ph[q] = p[q] / L.diag[q];
        apply_op(C, L, ph.data(), v.data());
        const double rv = dot(rh, v);
        if (rv == 0.0) break;
        alpha = rho / rv;
        for (size_t q = 0; q < N; ++q) s[q] = r[q] - alpha * v[q];
        if (norm_inf(s) <= tol) {
            for (size_t q = 0; q < N; ++q) x[q] += alpha * ph[q];
            break;
        }
        for (size_t q = 0; q < N; ++q) sh[q] = s[q] / L.diag[q];
        apply_op(C, L, sh.data(), t.data());
        const double tt = dot(t, t);
        omega = tt > 0.0 ? dot(t, s) / tt : 0.0;
        for (size_t q = 0; q < N; ++q) x[q] += alpha * ph[q] + omega * sh[q];
        for (size_t q = 0; q < N; ++q) r[q] = s[q] - omega * t[q];
        if (norm_inf(r) <= tol || omega == 0.0) break;
        rho_old = rho;
    }
}

void vcycle(Ctx& C, int l) {
    Level& L = C.lev[l];
    const int nlev = (int)C.lev.size();
    if (l == nlev - 1) {
        for (int s = 0; s < C.o.nub; ++s) gsrb(C, L);
        bottom_bicgstab(C, L);
        for (int s = 0; s < C.o.nub; ++s) gsrb(C, L);
        return;
    }
    for (int s = 0; s < C.o.nu1; ++s) gsrb(C, L);
    residual(C, L, L.phi.data(), L.f.data(), L.r.data());
    Level& K = C.lev[l + 1];
    restrict_defect(L, K);
    std::fill(K.phi.begin(), K.phi.end(), 0.0);
    vcycle(C, l + 1);
    prolong_add(C, K, L);
    for (int s = 0; s < C.o.nu2; ++s) gsrb(C, L);
}

// Build the level hierarchy from fine face coefficients (unscaled beta) and optional alpha.
void build_hierarchy(Ctx& C, const double* const b[3], const double* alpha) {
    const orc_opts& o = C.o;
    C.lev.assign(std::max(1, o.nlevels), Level());
    Level& F = C.lev[0];
    for (int d = 0; d < 3; ++d) {
        F.n[d] = o.n[d];
        F.h[d] = o.dx[d];
        F.act[d] = d < o.dm ? 1 : 0;
    }
    for (int d = 0; d < 3; ++d) {
        if (!F.act[d]) continue;
        const size_t m = (size_t)(F.n[0] + (d == 0)) * (F.n[1] + (d == 1)) * (F.n[2] + (d == 2));
        F.b[d].assign(b[d], b[d] + m);
    }
    if (alpha) F.alpha.assign(alpha, alpha + F.ncell());
    F.r.assign(F.ncell(), 0.0);
    build_diag(C, F);
    for (size_t l = 1; l < C.lev.size(); ++l) {
        coarsen_level(C, C.lev[l - 1], C.lev[l]);
        build_diag(C, C.lev[l]);
    }
    bool has_dir = false;
    for (int d = 0; d < o.dm; ++d)
        has_dir = has_dir || o.bc_lo[d] == ORC_BC_DIR || o.bc_hi[d] == ORC_BC_DIR;
    bool has_alpha = false;
    if (alpha)
        for (size_t q = 0; q < F.ncell(); ++q) has_alpha = has_alpha || alpha[q] != 0.0;
    C.singular = !has_dir && !has_alpha;
}

int solve(Ctx& C, const double* rh, double* phi, orc_stats* st) {
    Level& F = C.lev[0];
    F.f.assign(rh, rh + F.ncell());
    F.phi.assign(phi, phi + F.ncell());
    if (C.singular) sub_mean(F.f);
    const double fnorm = norm_inf(F.f);
    orc_stats local{};
    orc_stats& S = st ? *st : local;
    std::memset(&S, 0, sizeof(S));
    S.fnorm = fnorm;
    if (fnorm == 0.0) {
        std::fill(F.phi.begin(), F.phi.end(), 0.0);
        std::copy(F.phi.begin(), F.phi.end(), phi);
        return 0;
    }
    auto converged = [&](double res) {
        return res <= C.o.rel_eps * fnorm || (C.o.abs_eps > 0.0 && res <= C.o.abs_eps);
    };
    double res = residual(C, F, F.phi.data(), F.f.data(), nullptr);
    S.resid0 = res;
    int it = 0;
    while (!converged(res) && it < C.o.max_vcycles) {
        vcycle(C, 0);
        ++it;
        res = residual(C, F, F.phi.data(), F.f.data(), nullptr);
        if (S.nhist < 64) S.hist[S.nhist++] = res / fnorm;
    }
    S.vcycles = it;
    S.rel_resid = res / fnorm;
    S.status = converged(res) ? 0 : 1;
    S.bottom_iters = C.bottom_iters;
    std::copy(F.phi.begin(), F.phi.end(), phi);
    return S.status;
}

void set_threads(const orc_opts* o) {
#ifdef _OPENMP
    if (o->nthreads > 0) omp_set_num_threads(o->nthreads);
#else
    (void)o;
#endif
}

}  // namespace orc

using namespace orc;

extern "C" {

// Solve (alpha - div beta grad) phi = rh on one level with face coefficients b[d] (natural face
// layout, n[d]+1 faces along d).  phi is the initial guess on entry.  Mirrors mac_multigrid
// (Source/mac_multigrid.f90:18-67) with the MAC parameters.
int orc_mac_multigrid(const orc_opts* o, const double* rh, double* phi, const double* bx,
                      const double* by, const double* bz, const double* alpha, orc_stats* st) {
    set_threads(o);
    Ctx C;
    C.o = *o;
    const double* b[3] = {bx, by, bz};
    build_hierarchy(C, b, alpha);
    return solve(C, rh, phi, st);
}

// Apply (alpha - div beta grad) to u on the finest level.
void orc_apply_op(const orc_opts* o, const double* u, const double* bx, const double* by,
                  const double* bz, const double* alpha, double* out) {
    set_threads(o);
    Ctx C;
    C.o = *o;
    C.o.nlevels = 1;
    const double* b[3] = {bx, by, bz};
    build_hierarchy(C, b, alpha);
    apply_op(C, C.lev[0], u, out);
}

// Face coefficients of the MAC solve: beta_f = beta0^p * 2 / (rho_L + rho_R)
// (Source/macproject.f90:182-203, 698-738).  Ghost density: periodic wrap, otherwise the
// boundary cell value (first-order extrapolation of the density state).
void orc_mac_coeffs(const orc_opts* o, const double* rho, const double* beta0,
                    const double* beta0_edge, double* bx, double* by, double* bz) {
    set_threads(o);
    const int* n = o->n;
    const int va = o->dm - 1;
    double* b[3] = {bx, by, bz};
    for (int d = 0; d < o->dm; ++d) {
        const int m[3] = {n[0] + (d == 0), n[1] + (d == 1), n[2] + (d == 2)};
#pragma omp parallel for schedule(static)
        for (int k = 0; k < m[2]; ++k)
            for (int j = 0; j < m[1]; ++j)
                for (int i = 0; i < m[0]; ++i) {
                    int hi[3] = {i, j, k}, lo[3] = {i, j, k};
                    lo[d] -= 1;
                    auto fix = [&](int* q) {
                        if (q[d] < 0) q[d] = o->bc_lo[d] == ORC_BC_PER ? n[d] - 1 : 0;
                        if (q[d] >= n[d]) q[d] = o->bc_hi[d] == ORC_BC_PER ? 0 : n[d] - 1;
                    };
                    fix(hi);
                    fix(lo);
                    double v = 2.0 / (rho[cidx(n, hi[0], hi[1], hi[2])] + rho[cidx(n, lo[0], lo[1], lo[2])]);
                    if (beta0) {
                        const int r = (va == 0 ? i : va == 1 ? j : k);
                        const double bb = (d == va) ? beta0_edge[r] : beta0[r];
                        v *= bb;
                        if (o->alt_energy_fix) v *= bb;
                    }
                    b[d][fidx(n, d, i, j, k)] = v;
                }
    }
}

}  // extern "C"

namespace {

// Full MAC projection on one level (Source/macproject.f90:51-328), natural layout: u[d] has
// n[d]+1 faces along d; phi is the in/out initial guess; rho is the cell density; macrhs
// (nullable) the cell source.  The beta0 of face (d, i, j, k) comes from b0face (null: no beta0):
// the 1-D arrays for planar geometry (mult_edge_by_1d_coeff), the 3-D face multifab
// beta0_cart_edge for spherical geometry (multifab_mult_mult / multifab_div_div,
// Source/macproject.f90:155-161, 194-201, 236-241).
template <class B0>
int macproject_impl(const orc_opts* o, double* const* u, double* phi, const double* rho,
                    const double* macrhs, bool have_b0, const B0& b0face, orc_stats* st) {
    set_threads(o);
    const int* n = o->n;
    const int dm = o->dm;
    const size_t N = (size_t)n[0] * n[1] * n[2];

    auto scale_edges = [&](bool mult) {
        if (!have_b0) return;
        for (int d = 0; d < dm; ++d) {
            const int m[3] = {n[0] + (d == 0), n[1] + (d == 1), n[2] + (d == 2)};
#pragma omp parallel for schedule(static)
            for (int k = 0; k < m[2]; ++k)
                for (int j = 0; j < m[1]; ++j)
                    for (int i = 0; i < m[0]; ++i) {
                        const size_t fi = fidx(n, d, i, j, k);
                        const double bb = b0face(d, fi, i, j, k);
                        double& x = u[d][fi];
                        x = mult ? x * bb : x / bb;
                    }
        }
    };
    scale_edges(true);

    // divumac: rh = div(beta0 U); rh = rh - macrhs; rh = -rh
    std::vector<double> rh(N);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n[2]; ++k)
        for (int j = 0; j < n[1]; ++j)
            for (int i = 0; i < n[0]; ++i) {
                double dv = 0.0;
                for (int d = 0; d < dm; ++d) {
                    int hi[3] = {i, j, k};
                    hi[d] += 1;
                    dv += (u[d][fidx(n, d, hi[0], hi[1], hi[2])] - u[d][fidx(n, d, i, j, k)]) / o->dx[d];
                }
                const size_t c = cidx(n, i, j, k);
                if (macrhs) dv = dv - macrhs[c];
                rh[c] = -dv;
            }

    // solver_beta = beta0^p / rho_face (mk_mac_coeffs, then the beta0 multiplies)
    std::vector<double> bf[3];
    for (int d = 0; d < 3; ++d)
        bf[d].assign(d < dm ? (size_t)(n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2)) : 1, 0.0);
    orc_mac_coeffs(o, rho, nullptr, nullptr, bf[0].data(), bf[1].data(), bf[2].data());
    if (have_b0)
        for (int d = 0; d < dm; ++d) {
            const int m[3] = {n[0] + (d == 0), n[1] + (d == 1), n[2] + (d == 2)};
#pragma omp parallel for schedule(static)
            for (int k = 0; k < m[2]; ++k)
                for (int j = 0; j < m[1]; ++j)
                    for (int i = 0; i < m[0]; ++i) {
                        const size_t fi = fidx(n, d, i, j, k);
                        const double bb = b0face(d, fi, i, j, k);
                        bf[d][fi] *= bb;
                        if (o->alt_energy_fix) bf[d][fi] *= bb;
                    }
        }

    Ctx C;
    C.o = *o;
    const double* bp[3] = {bf[0].data(), bf[1].data(), bf[2].data()};
    build_hierarchy(C, bp, nullptr);
    const int status = solve(C, rh.data(), phi, st);

    // mkumac: beta0 U -= beta_f * G phi on every face; Neumann faces keep their value,
    // Dirichlet faces use the ghost -phi_boundary.
    for (int d = 0; d < dm; ++d) {
        const int m[3] = {n[0] + (d == 0), n[1] + (d == 1), n[2] + (d == 2)};
#pragma omp parallel for schedule(static)
        for (int k = 0; k < m[2]; ++k)
            for (int j = 0; j < m[1]; ++j)
                for (int i = 0; i < m[0]; ++i) {
                    const int f[3] = {i, j, k};
                    const int q = f[d];
                    double g;
                    int hi[3] = {i, j, k}, lo[3] = {i, j, k};
                    lo[d] -= 1;
                    if (q > 0 && q < n[d]) {
                        g = (phi[cidx(n, hi[0], hi[1], hi[2])] - phi[cidx(n, lo[0], lo[1], lo[2])]) / o->dx[d];
                    } else if ((q == 0 && o->bc_lo[d] == ORC_BC_PER) || (q == n[d] && o->bc_hi[d] == ORC_BC_PER)) {
                        hi[d] = 0;
                        lo[d] = n[d] - 1;
                        g = (phi[cidx(n, hi[0], hi[1], hi[2])] - phi[cidx(n, lo[0], lo[1], lo[2])]) / o->dx[d];
                    } else if (q == 0) {
                        g = (o->bc_lo[d] == ORC_BC_DIR) ? 2.0 * phi[cidx(n, hi[0], hi[1], hi[2])] / o->dx[d] : 0.0;
                    } else {
                        g = (o->bc_hi[d] == ORC_BC_DIR) ? -2.0 * phi[cidx(n, lo[0], lo[1], lo[2])] / o->dx[d] : 0.0;
                    }
                    const size_t fi = fidx(n, d, i, j, k);
                    u[d][fi] = u[d][fi] - bf[d][fi] * g;
                }
    }
    scale_edges(false);
    return status;
}

}  // namespace

extern "C" {

// Planar geometry: beta0 (nr = n[dm-1]) and beta0_edge (nr+1), nullable together.
int orc_macproject(const orc_opts* o, double* ux, double* uy, double* uz, double* phi,
                   const double* rho, const double* macrhs, const double* beta0,
                   const double* beta0_edge, orc_stats* st) {
    const int va = o->dm - 1;
    double* u[3] = {ux, uy, uz};
    auto b0 = [&](int d, size_t, int i, int j, int k) {
        const int r = va == 0 ? i : va == 1 ? j : k;
        return (d == va) ? beta0_edge[r] : beta0[r];
    };
    return macproject_impl(o, u, phi, rho, macrhs, beta0 != nullptr, b0, st);
}

// Spherical geometry: beta0 given on every face (beta0_cart_edge, natural face layout, n[d]+1
// faces along d), b0x / b0y / b0z.
int orc_macproject_cart(const orc_opts* o, double* ux, double* uy, double* uz, double* phi,
                        const double* rho, const double* macrhs, const double* b0x,
                        const double* b0y, const double* b0z, orc_stats* st) {
    double* u[3] = {ux, uy, uz};
    const double* bc[3] = {b0x, b0y, b0z};
    auto b0 = [&](int d, size_t fi, int, int, int) { return bc[d][fi]; };
    return macproject_impl(o, u, phi, rho, macrhs, true, b0, st);
}

// beta0 cell -> edge (Source/cell_to_edge.f90:14-70), single level, no coarse-fine chunks.
void orc_cell_to_edge(int nr, const double* s0_cell, double* s0_edge) {
    for (int r = 0; r <= nr; ++r) {
        if (r == 0) {
            s0_edge[r] = s0_cell[r];
        } else if (r == 1) {
            s0_edge[r] = 0.5 * (s0_cell[r - 1] + s0_cell[r]);
        } else if (r == nr) {
            s0_edge[r] = s0_cell[r - 1];
        } else if (r == nr - 1) {
            s0_edge[r] = 0.5 * (s0_cell[r] + s0_cell[r - 1]);
        } else {
            const double tmp = 7.0 / 12.0 * (s0_cell[r] + s0_cell[r - 1]) -
                               1.0 / 12.0 * (s0_cell[r + 1] + s0_cell[r - 2]);
            const double lo = std::min(s0_cell[r], s0_cell[r - 1]);
            const double hi = std::max(s0_cell[r], s0_cell[r - 1]);
            s0_edge[r] = std::min(std::max(tmp, lo), hi);
        }
    }
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
