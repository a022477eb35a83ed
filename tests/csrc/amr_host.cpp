// Host execution of the library's multi-level MAC projection (TEST INFRASTRUCTURE ONLY).
//
// Runs the per-cell functions and the amr_solve / amr_project sequencing of
// maestro_gb300/csrc/mac_amr.cuh -- the code the CUDA kernels of mac_amr.cu launch -- with plain
// loops over the cells and faces of each level, so the library's composite arithmetic and cycle
// order can be checked against the oracle without a GPU.  The level-0 coarse correction (the
// library's own one-level FP64 V-cycle on the device) is stood in for by one V-cycle of the
// oracle's one-level multigrid; it only sets the convergence rate, not the converged answer.
//
// Built by tests/test_amr_host_exec.py with g++ (no CUDA involved).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "mac_amr.cuh"
#include "mac_oracle_core.h"

using namespace mac;

namespace {

// The multigrid half of the executor in precision T (FP64, or FP32 for the inner cycles of the
// mixed-precision solve).  Level geometry and masks are shared with the FP64 executor.
template <typename T>
struct HostMl {
    int nlev = 0;
    amr::Geo geo{};
    bool singular = false;
    int err = 0;
    std::vector<amr::LevT<T>> L;
    std::vector<std::vector<T>> store[amr::kNumBufs];
    std::vector<T*> bufp[amr::kNumBufs];
    std::vector<std::vector<T>> beta[3];
    // the level-0 correction: the one-level FP64 V-cycle (of the FP64 executor for T = float)
    struct Level0 {
        orc::Ctx* base = nullptr;
        bool singular = false;
    } l0;

    amr::LevT<T> lev(int l) const { return L[l]; }
    T* buf(int l, int which) const { return bufp[which][l]; }
    long ncell(int l) const { return amr::ncells(L[l]); }
    int error() const { return err; }

    void defect(int l, const T* uu, const T* cu, const T* f, T* r) {
        const amr::LevT<T> C = l ? L[l - 1] : L[l];
        for (long i = 0; i < ncell(l); ++i) amr::defect_cell(geo, L[l], C, i, uu, cu, f, r);
    }
    void gsrb(int l, T* uu, const T* f, int nu) {
        for (int s = 0; s < nu; ++s)
            for (int colour = 0; colour < 2; ++colour)
                for (long t = 0; t < amr::colour_threads(L[l]); ++t) {
                    const long i = amr::colour_cell(L[l], t, colour);
                    if (i >= 0) amr::gsrb_cell(geo, L[l], i, colour, uu, f);
                }
    }
    void reflux(int l, const T* uf, const T* uc, T* res) {
        for (long i = 0; i < ncell(l - 1); ++i) amr::reflux_cell(geo, L[l], L[l - 1], i, uf, uc, res);
    }
    void restrict_cov(int l, const T* fine, T* crse) {
        for (long i = 0; i < ncell(l - 1); ++i) amr::restrict_cell(geo, L[l], L[l - 1], i, fine, crse);
    }
    void prolong(int l, const T* uc, T* uf) {
        for (long i = 0; i < ncell(l); ++i) amr::prolong_cell(geo, L[l], L[l - 1], i, uc, uf);
    }
    void axpy3(int l, T* uu, const T* hold, const T* du) {
        for (long i = 0; i < ncell(l); ++i)
            if (amr::in_region(L[l], i)) uu[i] += hold[i] + du[i];
    }
    void add_region(int l, T* phi, const T* uu) {
        for (long i = 0; i < ncell(l); ++i)
            if (amr::in_region(L[l], i)) phi[i] += uu[i];
    }
    void zero(int l, T* x) { std::fill(x, x + ncell(l), (T)0); }
    void copy(int l, T* dst, const T* src) { std::copy(src, src + ncell(l), dst); }
    void swap_bufs(int l, int a, int b) { std::swap(bufp[a][l], bufp[b][l]); }

    double vol(int l) const {
        return L[l].h[0] * (geo.dm > 1 ? L[l].h[1] : 1.0) * (geo.dm > 2 ? L[l].h[2] : 1.0);
    }
    double valid_max(int which) {
        double mx = 0.0;
        bool nan = false;
        for (int l = 0; l < nlev; ++l)
            for (long i = 0; i < ncell(l); ++i)
                if (amr::is_valid(L[l], i)) {
                    const double a = buf(l, which)[i];
                    nan = nan || a != a;
                    mx = std::max(mx, std::fabs(a));
                }
        return nan ? NAN : mx;
    }
    double valid_mean(int which) {
        double s = 0.0, v = 0.0;
        for (int l = 0; l < nlev; ++l)
            for (long i = 0; i < ncell(l); ++i)
                if (amr::is_valid(L[l], i)) {
                    s += vol(l) * buf(l, which)[i];
                    v += vol(l);
                }
        return s / v;
    }
    void sub_valid(int which, double m) {
        for (int l = 0; l < nlev; ++l)
            for (long i = 0; i < ncell(l); ++i)
                if (amr::is_valid(L[l], i)) buf(l, which)[i] -= (T)m;
    }
    int level0_correction(const T* rhs, T* e) {
        orc::Level& B = l0.base->lev[0];
        B.f.assign(rhs, rhs + ncell(0));
        if (l0.singular) orc::sub_mean(B.f);
        B.phi.assign(B.f.size(), 0.0);
        orc::vcycle(*l0.base, 0);
        if (l0.singular) orc::sub_mean(B.phi);
        for (long i = 0; i < ncell(0); ++i) e[i] = (T)B.phi[i];
        return 0;
    }
};

struct HostExec : HostMl<double> {
    std::vector<std::vector<unsigned char>> mask;
    orc::Ctx base;
    orc_opts o{};
    HostMl<float>* v32 = nullptr;
    // this call's inputs
    double* const* u = nullptr;
    const double* const* rho = nullptr;
    const double* const* macrhs = nullptr;
    const double* const* b0 = nullptr;
    const double* const* b0e = nullptr;
    int alt = 0;

    int prepare_level0() {
        const double* b[3] = {beta[0][0].data(), beta[1][0].data(),
                              geo.dm == 3 ? beta[2][0].data() : nullptr};
        base = orc::Ctx();
        base.o = o;
        orc::build_hierarchy(base, b, nullptr);
        singular = base.singular;
        l0.base = &base;
        l0.singular = singular;
        if (v32) {
            v32->singular = singular;
            v32->l0.base = &base;
            v32->l0.singular = singular;
        }
        return 0;
    }
    void faces_to_single() {
        for (int l = 0; l < nlev; ++l)
            for (int d = 0; d < geo.dm; ++d)
                for (size_t i = 0; i < beta[d][l].size(); ++i) v32->beta[d][l][i] = (float)beta[d][l][i];
    }
    void to_single(int l, const double* x, float* y) {
        for (long i = 0; i < ncell(l); ++i) amr::to_single_cell(i, x, y);
    }
    void accumulate(int l, double* phi, const float* e) {
        for (long i = 0; i < ncell(l); ++i) amr::accumulate_cell(L[l], i, phi, e);
    }
    void scale_b0(int l, bool mult) {
        if (!b0) return;
        for (int d = 0; d < geo.dm; ++d) {
            double* x = u[3 * l + d];
            for (long i = 0; i < amr::nfaces(L[l], d); ++i) {
                int f[3];
                amr::face_coords(L[l], d, i, f);
                const double bb = amr::beta0_of_face(geo, d, f, b0[l], b0e[l]);
                x[i] = mult ? x[i] * bb : x[i] / bb;
            }
        }
    }
    void edge_restrict(int l) {
        for (int d = 0; d < geo.dm; ++d)
            for (long i = 0; i < amr::nfaces(L[l - 1], d); ++i)
                amr::edge_restrict_face(geo, L[l], L[l - 1], d, i, u[3 * (l - 1) + d], u[3 * l + d]);
    }
    void divergence(int l) {
        for (long i = 0; i < ncell(l); ++i)
            amr::divergence_cell(geo, L[l], i, u[3 * l], u[3 * l + 1],
                                 geo.dm == 3 ? u[3 * l + 2] : nullptr,
                                 macrhs ? macrhs[l] : nullptr, buf(l, amr::kRh));
    }
    void coeffs(int l) {
        for (int d = 0; d < geo.dm; ++d)
            for (long i = 0; i < amr::nfaces(L[l], d); ++i)
                amr::coeff_face(geo, L[l], d, i, rho[l], b0 ? b0[l] : nullptr,
                                b0 ? b0e[l] : nullptr, alt, beta[d][l].data());
    }
    void correct(int l) {
        const amr::Lev C = l ? L[l - 1] : L[l];
        const double* cphi = l ? buf(l - 1, amr::kPhi) : nullptr;
        for (int d = 0; d < geo.dm; ++d)
            for (long i = 0; i < amr::nfaces(L[l], d); ++i)
                amr::correct_face(geo, L[l], C, d, i, buf(l, amr::kPhi), cphi, beta[d][l].data(),
                                  u[3 * l + d]);
    }
};

// Level storage of one precision from the FP64 executor's geometry and masks.
template <typename T>
void build_levels(HostMl<T>& M, const HostExec& E0) {
    const HostExec& E = E0;
    const std::vector<amr::Lev> geom = E.L;   // (M may be E itself)
    M.nlev = E.nlev;
    M.geo = E.geo;
    M.L.assign(E.nlev, amr::LevT<T>{});
    for (int b = 0; b < amr::kNumBufs; ++b) {
        M.store[b].assign(E.nlev, {});
        M.bufp[b].assign(E.nlev, nullptr);
    }
    for (int d = 0; d < 3; ++d) M.beta[d].assign(E.nlev, {});
    for (int l = 0; l < E.nlev; ++l) {
        amr::LevT<T>& V = M.L[l];
        for (int d = 0; d < 3; ++d) {
            V.n[d] = geom[l].n[d];
            V.lo[d] = geom[l].lo[d];
            V.ext[d] = geom[l].ext[d];
            amr::set_spacing(V, d, geom[l].h[d]);
        }
        V.mask = E.mask[l].data();
        const long N = amr::ncells(V);
        // work arrays and coefficients start as NaN: the device arrays they stand for are not
        // initialised, so any read before a write shows up in the results
        const T nan = std::numeric_limits<T>::quiet_NaN();
        for (int b = 0; b < amr::kNumBufs; ++b) {
            M.store[b][l].assign((size_t)N, nan);
            M.bufp[b][l] = M.store[b][l].data();
        }
        for (int d = 0; d < E.geo.dm; ++d) M.beta[d][l].assign((size_t)amr::nfaces(V, d), nan);
        for (int d = 0; d < 3; ++d) V.b[d] = d < E.geo.dm ? M.beta[d][l].data() : nullptr;
    }
}

// Masks from the boxes (no layout validation here: the oracle's own checks cover it).
void build(HostExec& E, const orc_opts* o, int nlev, const int* nboxes, const int* boxes) {
    E.o = *o;
    E.nlev = nlev;
    E.geo.dm = o->dm;
    E.geo.va = o->dm - 1;
    for (int d = 0; d < 3; ++d) {
        E.geo.per[d] = o->bc_lo[d] == ORC_BC_PER;
        E.geo.dlo[d] = o->bc_lo[d] == ORC_BC_DIR;
        E.geo.dhi[d] = o->bc_hi[d] == ORC_BC_DIR;
    }
    E.L.assign(nlev, amr::Lev{});
    E.mask.assign(nlev, {});
    const int per[3] = {E.geo.per[0], E.geo.per[1], E.geo.per[2]};
    const int* bx = boxes;
    for (int l = 0; l < nlev; ++l) {
        amr::Lev& V = E.L[l];
        for (int d = 0; d < 3; ++d) {
            V.n[d] = d < o->dm ? (o->n[d] << l) : 1;
            amr::set_spacing(V, d, d < o->dm ? o->dx[d] / (double)(1 << l) : o->dx[d]);
            V.lo[d] = 0;
            V.ext[d] = V.n[d];
        }
        if (l > 0) {   // the bounding box of the level's boxes, grown by one cell
            int rlo[3] = {1 << 30, 1 << 30, 1 << 30}, rhi[3] = {-1, -1, -1};
            for (int b = 0; b < nboxes[l]; ++b)
                for (int d = 0; d < 3; ++d) {
                    rlo[d] = std::min(rlo[d], bx[6 * b + d]);
                    rhi[d] = std::max(rhi[d], bx[6 * b + 3 + d]);
                }
            amr::level_box(o->dm, V.n, per, rlo, rhi, V.lo, V.ext);
            bx += 6 * nboxes[l];
        }
        E.mask[l].assign((size_t)amr::ncells(V), l == 0 ? amr::kIn : 0);
    }
    bx = boxes;
    for (int l = 1; l < nlev; ++l)
        for (int b = 0; b < nboxes[l]; ++b, bx += 6)
            for (int k = bx[2]; k <= bx[5]; ++k)
                for (int j = bx[1]; j <= bx[4]; ++j)
                    for (int i = bx[0]; i <= bx[3]; ++i)
                        E.mask[l][amr::cix(E.L[l], i, j, k)] = amr::kIn;
    for (int l = 1; l < nlev; ++l)
        for (long i = 0; i < amr::ncells(E.L[l]); ++i) {
            if (!E.mask[l][i]) continue;
            int c[3];
            amr::cell_coords(E.L[l], i, c);
            int p[3];
            for (int d = 0; d < 3; ++d) p[d] = d < o->dm ? c[d] >> 1 : c[d];
            E.mask[l - 1][amr::cix(E.L[l - 1], p[0], p[1], p[2])] |= amr::kCov;
        }
    for (int l = 0; l < nlev; ++l) E.L[l].mask = E.mask[l].data();
    build_levels<double>(E, E);
}

}  // namespace

extern "C" {

// Cell, colour and face coordinates of a level array box (the 32-bit index arithmetic of
// mac_amr.cuh) against plain 64-bit arithmetic on every index: the number of mismatches.
long amrh_coords_check(const int* lo, const int* ext) {
    amr::Lev L{};
    for (int d = 0; d < 3; ++d) {
        L.lo[d] = lo[d];
        L.ext[d] = ext[d];
        L.n[d] = lo[d] + ext[d];
    }
    long bad = 0;
    const long nc = (long)ext[0] * ext[1] * ext[2];
    for (long idx = 0; idx < nc; ++idx) {
        int c[3];
        amr::cell_coords(L, idx, c);
        const long r = idx / ext[0];
        bad += c[0] != lo[0] + (int)(idx % ext[0]) || c[1] != lo[1] + (int)(r % ext[1]) ||
               c[2] != lo[2] + (int)(r / ext[1]);
    }
    for (int d = 0; d < 3; ++d) {
        const long m0 = ext[0] + (d == 0), m1 = ext[1] + (d == 1), m2 = ext[2] + (d == 2);
        for (long idx = 0; idx < m0 * m1 * m2; ++idx) {
            int f[3];
            amr::face_coords(L, d, idx, f);
            const long r = idx / m0;
            bad += f[0] != lo[0] + (int)(idx % m0) || f[1] != lo[1] + (int)(r % m1) ||
                   f[2] != lo[2] + (int)(r / m1);
        }
    }
    const long hw = (ext[0] + 1) / 2;
    for (int colour = 0; colour < 2; ++colour)
        for (long t = 0; t < amr::colour_threads(L); ++t) {
            const long row = t / hw;
            const int j = (int)(row % ext[1]), k = (int)(row / ext[1]);
            const int x0 = (colour + lo[0] + lo[1] + j + lo[2] + k) & 1;
            const int x = 2 * (int)(t % hw) + x0;
            const long want = x >= ext[0] ? -1 : (long)x + (long)ext[0] * ((long)j + (long)ext[1] * k);
            bad += amr::colour_cell(L, t, colour) != want;
        }
    return bad;
}

// The library's multi-level projection run on the host; arguments as orc_macproject_ml
// (phi[l] in/out, umac[3 l + d] in/out).  Returns the solve status (0 converged).
int amrh_macproject_prec(const orc_opts* o, int nlev, const int* nboxes, const int* boxes,
                         double* const* umac, double* const* phi, const double* const* rho,
                         const double* const* macrhs, const double* const* beta0,
                         const double* const* beta0_edge, int inner, int fab_inputs,
                         double* stats_out);

int amrh_macproject(const orc_opts* o, int nlev, const int* nboxes, const int* boxes,
                    double* const* umac, double* const* phi, const double* const* rho,
                    const double* const* macrhs, const double* const* beta0,
                    const double* const* beta0_edge, double* stats_out) {
    return amrh_macproject_prec(o, nlev, nboxes, boxes, umac, phi, rho, macrhs, beta0,
                                beta0_edge, 0, 0, stats_out);
}

// inner > 0: the mixed-precision solve, `inner` FP32 multi-level V-cycles per FP64 step.
// fab_inputs: the fine levels' input arrays hold only what the per-box entry gathers from fabs
// (each box's own faces and cells, density ghosts one cell deep); everything else is NaN, as
// the uninitialised device arrays of that entry.
int amrh_macproject_prec(const orc_opts* o, int nlev, const int* nboxes, const int* boxes,
                         double* const* umac, double* const* phi, const double* const* rho,
                         const double* const* macrhs, const double* const* beta0,
                         const double* const* beta0_edge, int inner, int fab_inputs,
                         double* stats_out) {
    HostExec E;
    build(E, o, nlev, nboxes, boxes);
    HostMl<float> E32;
    build_levels<float>(E32, E);
    E.v32 = &E32;
    // the caller's whole-level-domain arrays -> the levels' box arrays
    const int dm = o->dm;
    std::vector<std::vector<double>> ub(3 * nlev), rb(nlev), mb(nlev);
    std::vector<double*> up(3 * nlev, nullptr);
    std::vector<const double*> rp(nlev), mp(nlev, nullptr);
    for (int l = 0; l < nlev; ++l) {
        const amr::Lev& V = E.L[l];
        for (int d = 0; d < dm; ++d) {
            ub[3 * l + d].resize((size_t)amr::nfaces(V, d));
            for (long i = 0; i < amr::nfaces(V, d); ++i)
                ub[3 * l + d][i] = umac[3 * l + d][amr::full_face(V, d, i)];
            up[3 * l + d] = ub[3 * l + d].data();
        }
        rb[l].resize((size_t)amr::ncells(V));
        for (long i = 0; i < amr::ncells(V); ++i) {
            rb[l][i] = rho[l][amr::full_cell(V, i)];
            E.buf(l, amr::kPhi)[i] = phi[l][amr::full_cell(V, i)];
        }
        rp[l] = rb[l].data();
        if (macrhs && macrhs[l]) {
            mb[l].resize((size_t)amr::ncells(V));
            for (long i = 0; i < amr::ncells(V); ++i) mb[l][i] = macrhs[l][amr::full_cell(V, i)];
            mp[l] = mb[l].data();
        }
    }
    if (fab_inputs) {
        const double nan = std::numeric_limits<double>::quiet_NaN();
        const int* bx = boxes;
        for (int l = 1; l < nlev; ++l) {
            const amr::Lev& V = E.L[l];
            std::vector<char> face_set[3], cell_set((size_t)amr::ncells(V), 0),
                rho_set((size_t)amr::ncells(V), 0);
            for (int d = 0; d < dm; ++d) face_set[d].assign((size_t)amr::nfaces(V, d), 0);
            for (int b = 0; b < nboxes[l]; ++b, bx += 6) {
                for (int dir = -1; dir < dm; ++dir) {
                    amr::FabDesc D{};
                    long cnt = 1;
                    for (int d = 0; d < 3; ++d) {
                        D.lo[d] = bx[d];
                        D.hi[d] = bx[3 + d];
                        D.ext[d] = d < dm ? D.hi[d] - D.lo[d] + 1 + (dir == d) + 2 : 1;
                        cnt *= D.ext[d];
                    }
                    D.ng = 1;
                    D.count = cnt;
                    for (long e = 0; e < cnt; ++e) {
                        long t;
                        const int kind = amr::fab_elem(E.geo, V, dir, D, e, &t);
                        if (dir >= 0 && kind == 1) face_set[dir][t] = 1;
                        if (dir < 0 && kind == 1) cell_set[t] = 1;
                        if (dir < 0 && kind >= 1) rho_set[t] = 1;
                    }
                }
            }
            for (int d = 0; d < dm; ++d) {
                for (long i = 0; i < amr::nfaces(V, d); ++i)
                    if (!face_set[d][i]) ub[3 * l + d][i] = nan;
                const long nt = amr::ncells(V) / V.ext[d];
                for (long t = 0; t < nt; ++t) amr::sync_periodic_face(E.geo, V, d, t, ub[3 * l + d].data());
            }
            for (long i = 0; i < amr::ncells(V); ++i) {
                if (!rho_set[i]) rb[l][i] = nan;
                if (!cell_set[i]) {
                    E.buf(l, amr::kPhi)[i] = nan;
                    if (mp[l]) mb[l][i] = nan;
                }
            }
        }
    }
    E.u = up.data();
    E.rho = rp.data();
    E.macrhs = macrhs ? mp.data() : nullptr;
    E.b0 = beta0;
    E.b0e = beta0_edge;
    E.alt = o->alt_energy_fix;
    amr::SolveStats S{};
    const int rc = amr::amr_project(E, o->rel_eps, o->abs_eps, o->max_vcycles, o->nu1, o->nu2,
                                    &S, inner > 0 ? &E32 : nullptr, inner);
    // back: the levels' own faces and region cells
    for (int l = 0; l < nlev; ++l) {
        const amr::Lev& V = E.L[l];
        for (int d = 0; d < dm; ++d)
            for (long i = 0; i < amr::nfaces(V, d); ++i) {
                int f[3];
                amr::face_coords(V, d, i, f);
                if (amr::face_in_level(E.geo, V, d, f))
                    umac[3 * l + d][amr::full_face(V, d, i)] = ub[3 * l + d][i];
            }
        for (long i = 0; i < amr::ncells(V); ++i)
            if (amr::in_region(V, i)) phi[l][amr::full_cell(V, i)] = E.buf(l, amr::kPhi)[i];
    }
    if (stats_out) {
        stats_out[0] = rc;
        stats_out[1] = S.cycles;
        stats_out[2] = S.rel_resid;
        stats_out[3] = S.fnorm;
    }
    return rc;
}


// Caller fabs <-> a level array with the library's fab functions.  fabs[b] are the fab images of
// level l's boxes (level 0: the single domain box is not used; l >= 1), dir the face direction
// (-1 cells).  gather: level += nothing, entries set from the fabs; scatter: fab entries of the
// boxes set from the level array.
void amrh_fabs(const orc_opts* o, int nlev, const int* nboxes, const int* boxes, int l, int dir,
               int ng, int with_ghosts, int scatter, double* const* fabs, double* level) {
    HostExec E;
    build(E, o, nlev, nboxes, boxes);
    const amr::Lev& V = E.L[l];
    // the whole-level-domain array of the caller <-> the level's box array
    const long nbox = dir < 0 ? amr::ncells(V) : amr::nfaces(V, dir);
    std::vector<double> box((size_t)nbox, 0.0);
    auto full = [&](long i) { return dir < 0 ? amr::full_cell(V, i) : amr::full_face(V, dir, i); };
    if (scatter)
        for (long i = 0; i < nbox; ++i) box[i] = level[full(i)];
    const int* bx = boxes;
    for (int q = 1; q < l; ++q) bx += 6 * nboxes[q];
    for (int b = 0; b < nboxes[l]; ++b, bx += 6) {
        amr::FabDesc D{};
        long cnt = 1;
        for (int d = 0; d < 3; ++d) {
            D.lo[d] = bx[d];
            D.hi[d] = bx[3 + d];
            D.ext[d] = d < o->dm ? D.hi[d] - D.lo[d] + 1 + (dir == d) + 2 * ng : 1;
            cnt *= D.ext[d];
        }
        D.ng = ng;
        D.count = cnt;
        D.src = fabs[b];
        D.dst = fabs[b];
        for (long e = 0; e < cnt; ++e) {
            if (scatter)
                amr::fab_scatter_elem(E.geo, V, dir, D, e, box.data());
            else
                amr::fab_gather_elem(E.geo, V, dir, D, e, with_ghosts, box.data());
        }
    }
    if (!scatter)
        for (long i = 0; i < nbox; ++i) level[full(i)] = box[i];
}

// The colour map of the smoother launches over a box lo[3], ext[3] (dm active directions):
// returns 0 when every cell of each colour is hit exactly once and nothing else is.
int amrh_check_colour_map(int dm, const int* lo, const int* ext) {
    amr::Lev L{};
    for (int d = 0; d < 3; ++d) {
        L.lo[d] = d < dm ? lo[d] : 0;
        L.ext[d] = d < dm ? ext[d] : 1;
    }
    for (int colour = 0; colour < 2; ++colour) {
        std::vector<int> hits((size_t)amr::ncells(L), 0);
        for (long t = 0; t < amr::colour_threads(L); ++t) {
            const long i = amr::colour_cell(L, t, colour);
            if (i < -1 || i >= amr::ncells(L)) return 1;
            if (i >= 0) ++hits[(size_t)i];
        }
        for (long i = 0; i < amr::ncells(L); ++i) {
            int c[3];
            amr::cell_coords(L, i, c);
            const int want = ((c[0] + c[1] + c[2]) & 1) == colour ? 1 : 0;
            if (hits[(size_t)i] != want) return 2;
        }
    }
    return 0;
}

}  // extern "C"
