// Host execution of the library's nodal (HG) projection (TEST INFRASTRUCTURE ONLY).
//
// Runs the node / cell functions and the hg::project / hg::solve / hg::vcycle sequencing of
// maestro_gb300/csrc/hg_nodal.cuh -- the code the CUDA kernels of hg_nodal.cu launch -- with
// loops over the nodes and cells, so the nodal arithmetic and the cycle order are checked without
// a GPU.  Built by tests/test_hg_host_exec.py with g++ (no CUDA involved).
#include <algorithm>
#include <cmath>
#include <vector>

#include "hg_nodal.cuh"

using namespace mac;

namespace {

struct HostLevel {
    hg::Lev lev{};
    std::vector<double> sig;
    std::vector<double> buf[hg::kNumBufs];
};

struct HostExec {
    int nlev = 0;
    hg::Geo geo{};
    bool singular = true;
    std::vector<HostLevel> L;
    double last_mean = 0.0;
    int proj_type = hg::kRegular;
    double dt = 1.0;
    double* unew = nullptr;
    const double* uold = nullptr;
    double* gpi = nullptr;
    const double* rhohalf = nullptr;
    double* pi = nullptr;
    const double* b0 = nullptr;
    const double* nodalrhs = nullptr;
    int alt = 0;

    hg::Lev lev(int l) const { return L[l].lev; }
    double* buf(int l, int w) { return L[l].buf[w].data(); }
    long nn(int l) const { return hg::nnodes(L[l].lev); }
    long nc(int l) const { return hg::ncells(L[l].lev); }
    int error() const { return 0; }

    void defect(int l, const double* phi, const double* f, double* r) {
        for (long i = 0; i < nn(l); ++i) hg::defect_node(geo, L[l].lev, i, phi, f, r);
    }
    void gs(int l, double* phi, const double* f, int nu) {
        for (int s = 0; s < nu; ++s)
            for (int colour = 0; colour < (1 << geo.dm); ++colour) {
                const long m = hg::colour_count(geo, L[l].lev, colour);
                for (long i = 0; i < m; ++i) hg::gs_node(geo, L[l].lev, i, colour, phi, f);
            }
    }
    void bottom_gs(int l, double* phi, const double* f, int nu) { gs(l, phi, f, nu); }
    void restrict_to(int lc, const double* rF, double* fK) {
        for (long i = 0; i < nn(lc); ++i) hg::restrict_node(geo, L[lc - 1].lev, L[lc].lev, i, rF, fK);
    }
    void prolong(int lc, const double* eK, double* phiF) {
        for (long i = 0; i < nn(lc - 1); ++i) hg::prolong_node(geo, L[lc].lev, L[lc - 1].lev, i, eK, phiF);
    }
    void zero(int l, double* x) { std::fill(x, x + nn(l), 0.0); }
    void finish(int l, double* x) {
        for (long i = 0; i < nn(l); ++i) hg::finish_node(geo, L[l].lev, i, x);
    }
    double unknown_max(int l, const double* x) {
        double mx = 0.0;
        bool nan = false;
        for (long i = 0; i < nn(l); ++i) {
            int p[3];
            hg::node_coords(L[l].lev, i, p);
            if (!hg::is_unknown(geo, L[l].lev, p)) continue;
            nan = nan || x[i] != x[i];
            mx = std::max(mx, std::fabs(x[i]));
        }
        return nan ? NAN : mx;
    }
    void sub_unknown_mean(int l, double* x) {
        double s = 0.0;
        long cnt = 0;
        for (long i = 0; i < nn(l); ++i) {
            int p[3];
            hg::node_coords(L[l].lev, i, p);
            if (!hg::is_unknown(geo, L[l].lev, p)) continue;
            s += x[i];
            ++cnt;
        }
        const double m = cnt ? s / cnt : 0.0;
        for (long i = 0; i < nn(l); ++i) {
            int p[3];
            hg::node_coords(L[l].lev, i, p);
            if (hg::is_unknown(geo, L[l].lev, p)) x[i] -= m;
        }
    }
    void uvec() {
        for (long i = 0; i < nc(0); ++i)
            hg::uvec_cell(geo, i, nc(0), proj_type, dt, unew, uold, gpi, rhohalf, b0, alt, L[0].sig.data());
    }
    int build_levels() {
        for (int l = 1; l < nlev; ++l)
            for (long i = 0; i < nc(l); ++i)
                hg::coarsen_sig_cell(geo, L[l - 1].lev, L[l].lev, i, L[l].sig.data());
        return 0;
    }
    void divu() {
        for (long i = 0; i < nn(0); ++i)
            hg::divu_node(geo, L[0].lev, i, unew, b0, nodalrhs, buf(0, hg::kF));
    }
    void update() {
        for (long i = 0; i < nc(0); ++i)
            hg::update_cell(geo, L[0].lev, i, proj_type, dt, buf(0, hg::kPhi), unew, uold, gpi,
                            rhohalf, b0, alt);
        for (long i = 0; i < nn(0); ++i)
            hg::update_pi_node(L[0].lev, i, proj_type, dt, buf(0, hg::kPhi), pi);
    }
};

}  // namespace

extern "C" {

// The library's nodal projection on the host.  Geometry: dm, n[3], dx[3], per/dlo/dhi flags;
// arrays as mac_hgproject_dense.  phi_out (nullable) receives the nodal solution.  stats_out:
// [status, cycles, rel_resid, fnorm].
int hgh_project(int dm, const int* n, const double* dx, const int* per, const int* dlo,
                const int* dhi, int dense, int proj_type, double dt, int alt, double rel_eps,
                int max_cycles, int nu1, int nu2, double* unew, const double* uold, double* gpi,
                const double* rhohalf, double* pi, const double* b0, const double* nodalrhs,
                double* phi_out, double* stats_out) {
    HostExec E;
    E.geo.dm = dm;
    for (int d = 0; d < 3; ++d) {
        E.geo.per[d] = d < dm ? per[d] : 0;
        E.geo.dlo[d] = d < dm ? dlo[d] : 0;
        E.geo.dhi[d] = d < dm ? dhi[d] : 0;
    }
    E.geo.dense = dense;
    bool dir = false;
    for (int d = 0; d < dm; ++d) dir = dir || E.geo.dlo[d] || E.geo.dhi[d];
    E.singular = !dir;
    int nn[3];
    double h[3];
    for (int d = 0; d < 3; ++d) {
        nn[d] = d < dm ? n[d] : 1;
        h[d] = d < dm ? dx[d] : 1.0;
    }
    while (true) {
        HostLevel S;
        for (int d = 0; d < 3; ++d) {
            S.lev.n[d] = nn[d];
            S.lev.nn[d] = d < dm ? nn[d] + 1 : 1;
            S.lev.h[d] = h[d];
        }
        S.sig.assign((size_t)hg::ncells(S.lev), 0.0);
        for (int b = 0; b < hg::kNumBufs; ++b) S.buf[b].assign((size_t)hg::nnodes(S.lev), 0.0);
        E.L.push_back(std::move(S));
        bool more = (int)E.L.size() < hg::kMaxLevels;
        for (int d = 0; d < dm; ++d) more = more && nn[d] % 2 == 0 && nn[d] >= 4;
        if (!more) break;
        for (int d = 0; d < dm; ++d) {
            nn[d] /= 2;
            h[d] *= 2;
        }
    }
    for (HostLevel& S : E.L) {
        S.lev.sig = S.sig.data();
        hg::set_dense_weights(dm, S.lev);
    }
    E.nlev = (int)E.L.size();
    E.proj_type = proj_type;
    E.dt = dt;
    E.unew = unew;
    E.uold = uold;
    E.gpi = gpi;
    E.rhohalf = rhohalf;
    E.pi = pi;
    E.b0 = b0;
    E.nodalrhs = nodalrhs;
    E.alt = (proj_type != hg::kInitial && proj_type != hg::kDivuIters && alt) ? 1 : 0;
    hg::SolveStats S{};
    const int rc = hg::project(E, rel_eps, max_cycles, nu1, nu2, &S);
    if (phi_out) std::copy(E.L[0].buf[hg::kPhi].begin(), E.L[0].buf[hg::kPhi].end(), phi_out);
    if (stats_out) {
        stats_out[0] = rc;
        stats_out[1] = S.cycles;
        stats_out[2] = S.rel_resid;
        stats_out[3] = S.fnorm;
    }
    return rc;
}


// Caller fabs <-> a whole-domain cell / node array with the library's fab mapping; boxes as
// lo[3], hi[3] per box; scatter: fabs <- array, else array <- fabs.
void hgh_fabs(int dm, const int* n, const int* per, int nboxes, const int* boxes, int ng,
              int nodal, int ncomp, int scatter, double* const* fabs, double* arr) {
    hg::Geo G{};
    G.dm = dm;
    for (int d = 0; d < 3; ++d) G.per[d] = d < dm ? per[d] : 0;
    hg::Lev L{};
    for (int d = 0; d < 3; ++d) {
        L.n[d] = d < dm ? n[d] : 1;
        L.nn[d] = d < dm ? n[d] + 1 : 1;
        L.h[d] = 1.0;
    }
    const long stride = nodal ? hg::nnodes(L) : hg::ncells(L);
    for (int b = 0; b < nboxes; ++b) {
        hg::Fab F{};
        long cnt = 1;
        for (int d = 0; d < 3; ++d) {
            F.lo[d] = boxes[6 * b + d];
            F.hi[d] = boxes[6 * b + 3 + d];
            F.ext[d] = d < dm ? F.hi[d] - F.lo[d] + 1 + nodal + 2 * ng : 1;
            cnt *= F.ext[d];
        }
        F.ng = ng;
        F.nodal = nodal;
        F.count = cnt;
        for (long e = 0; e < cnt; ++e) {
            const long t = hg::fab_target(G, L, F, e);
            if (t < 0) continue;
            for (int q = 0; q < ncomp; ++q) {
                if (scatter)
                    fabs[b][q * cnt + e] = arr[q * stride + t];
                else
                    arr[q * stride + t] = fabs[b][q * cnt + e];
            }
        }
    }
}

}  // extern "C"
