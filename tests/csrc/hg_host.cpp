// Host execution of the library's nodal (HG) projection (TEST INFRASTRUCTURE ONLY).
//
// Runs the node / cell functions and the hg::project / hg::solve / hg::vcycle sequencing of
// maestro_gb300/csrc/hg_nodal.cuh -- the code the CUDA kernels of hg_nodal.cu launch -- with
// loops over the nodes and cells, so the nodal arithmetic and the cycle order are checked without
// a GPU.  Built by tests/test_hg_host_exec.py with g++ (no CUDA involved).
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "hg_nodal.cuh"

using namespace mac;

namespace {

// The multigrid half of the executor in precision T (FP64, or FP32 for the inner cycles).
template <typename T>
struct HostMg {
    int nlev = 0;
    hg::Geo geo{};
    bool singular = true;
    std::vector<hg::LevT<T>> L;
    std::vector<std::vector<T>> sig;
    std::vector<std::vector<T>> store[hg::kNumBufs];

    void build(const hg::Geo& G, bool sing, const std::vector<hg::LevT<double>>& shape) {
        geo = G;
        singular = sing;
        nlev = (int)shape.size();
        L.assign(nlev, hg::LevT<T>{});
        sig.assign(nlev, {});
        for (int b = 0; b < hg::kNumBufs; ++b) store[b].assign(nlev, {});
        // work arrays start as NaN: the device arrays they stand for are not initialised, so
        // any read before a write shows up in the results
        const T nan = std::numeric_limits<T>::quiet_NaN();
        for (int l = 0; l < nlev; ++l) {
            for (int d = 0; d < 3; ++d) {
                L[l].n[d] = shape[l].n[d];
                L[l].nn[d] = shape[l].nn[d];
                L[l].h[d] = shape[l].h[d];
            }
            sig[l].assign((size_t)hg::ncells(L[l]), nan);
            for (int b = 0; b < hg::kNumBufs; ++b) store[b][l].assign((size_t)hg::nnodes(L[l]), nan);
            L[l].sig = sig[l].data();
            hg::set_dense_weights(geo.dm, L[l]);
        }
    }
    hg::LevT<T> lev(int l) const { return L[l]; }
    T* buf(int l, int w) { return store[w][l].data(); }
    long nn(int l) const { return hg::nnodes(L[l]); }
    long nc(int l) const { return hg::ncells(L[l]); }
    int error() const { return 0; }

    void defect(int l, const T* phi, const T* f, T* r) {
        for (long i = 0; i < nn(l); ++i) hg::defect_node(geo, L[l], i, phi, f, r);
    }
    void gs(int l, T* phi, const T* f, int nu) {
        for (int s = 0; s < nu; ++s)
            for (int colour = 0; colour < (1 << geo.dm); ++colour) {
                const long m = hg::colour_count(geo, L[l], colour);
                for (long i = 0; i < m; ++i) hg::gs_node(geo, L[l], i, colour, phi, f);
            }
    }
    void bottom_gs(int l, T* phi, const T* f, int nu) { gs(l, phi, f, nu); }
    void restrict_to(int lc, const T* rF, T* fK) {
        for (long i = 0; i < nn(lc); ++i) hg::restrict_node(geo, L[lc - 1], L[lc], i, rF, fK);
    }
    void prolong(int lc, const T* eK, T* phiF) {
        for (long i = 0; i < nn(lc - 1); ++i) hg::prolong_node(geo, L[lc], L[lc - 1], i, eK, phiF);
    }
    void zero(int l, T* x) { std::fill(x, x + nn(l), (T)0); }
    void finish(int l, T* x) {
        for (long i = 0; i < nn(l); ++i) hg::finish_node(geo, L[l], i, x);
    }
    double unknown_max(int l, const T* x) {
        double mx = 0.0;
        bool nan = false;
        for (long i = 0; i < nn(l); ++i) {
            int p[3];
            hg::node_coords(L[l], i, p);
            if (!hg::is_unknown(geo, L[l], p)) continue;
            nan = nan || x[i] != x[i];
            mx = std::max(mx, (double)std::fabs(x[i]));
        }
        return nan ? NAN : mx;
    }
    void sub_unknown_mean(int l, T* x) {
        double s = 0.0;
        long cnt = 0;
        for (long i = 0; i < nn(l); ++i) {
            int p[3];
            hg::node_coords(L[l], i, p);
            if (!hg::is_unknown(geo, L[l], p)) continue;
            s += x[i];
            ++cnt;
        }
        const T m = (T)(cnt ? s / cnt : 0.0);
        for (long i = 0; i < nn(l); ++i) {
            int p[3];
            hg::node_coords(L[l], i, p);
            if (hg::is_unknown(geo, L[l], p)) x[i] -= m;
        }
    }
};

// FP64 executor: the multigrid plus the projection steps and the precision hand-over.
struct HostExec : HostMg<double> {
    HostMg<float>* v32 = nullptr;
    int proj_type = hg::kRegular;
    double dt = 1.0;
    double* unew = nullptr;
    const double* uold = nullptr;
    double* gpi = nullptr;
    const double* rhohalf = nullptr;
    double* pi = nullptr;
    const double* b0 = nullptr;
    const double* nodalrhs = nullptr;
    hg::Wall wall{nullptr, {-1, -1, -1, -1, -1, -1}};
    int alt = 0;

    void uvec() {
        for (long i = 0; i < nc(0); ++i)
            hg::uvec_cell(geo, i, nc(0), proj_type, dt, 1.0 / dt, unew, uold, gpi, rhohalf, b0, alt,
                          sig[0].data());
    }
    int build_levels() {
        for (int l = 1; l < nlev; ++l)
            for (long i = 0; i < nc(l); ++i) hg::coarsen_sig_cell(geo, L[l - 1], L[l], i, sig[l].data());
        return 0;
    }
    void sig_to_single() {
        for (int l = 0; l < nlev; ++l)
            for (long i = 0; i < nc(l); ++i) v32->sig[l][i] = (float)sig[l][i];
    }
    void to_single(const double* r, float* r32) {
        for (long i = 0; i < nn(0); ++i) hg::to_single_node(i, r, r32);
    }
    void accumulate(double* phi, const float* e) {
        for (long i = 0; i < nn(0); ++i) hg::accumulate_node(geo, L[0], i, phi, e);
    }
    void divu() {
        for (long i = 0; i < nn(0); ++i)
            hg::divu_node(geo, L[0], i, unew, b0, nodalrhs, wall, buf(0, hg::kF));
    }
    void update() {
        for (long i = 0; i < nc(0); ++i)
            hg::update_cell(geo, L[0], i, proj_type, dt, 1.0 / dt, buf(0, hg::kPhi), unew, uold,
                            gpi, rhohalf, b0, alt);
        for (long i = 0; i < nn(0); ++i)
            hg::update_pi_node(L[0], i, proj_type, dt, buf(0, hg::kPhi), pi);
    }
};

// inflow faces of the next projection (hgh_set_wall)
hg::Wall g_wall{nullptr, {-1, -1, -1, -1, -1, -1}};

}  // namespace

extern "C" {

// The dense stencil's weight table (set_dense_weights) of a level with spacing h, in FP64 and
// as the FP32 levels hold it: kw64[8], kw32[8].
void hgh_dense_weights(int dm, const double* h, double* kw64, float* kw32) {
    hg::LevT<double> L{};
    hg::LevT<float> L32{};
    for (int d = 0; d < 3; ++d) L.h[d] = L32.h[d] = h[d];
    hg::set_dense_weights(dm, L);
    hg::set_dense_weights(dm, L32);
    for (int x = 0; x < 8; ++x) {
        kw64[x] = L.kw[x];
        kw32[x] = L32.kw[x];
    }
}

// Inflow faces for the following hgh_project* calls: off[f] >= 0 marks face f = 2 d + side as an
// inflow face with its wall values at w + off[f] (hg::Wall); off NULL: none.
void hgh_set_wall(const long* off, const double* w) {
    g_wall.w = off ? w : nullptr;
    for (int f = 0; f < 6; ++f) g_wall.off[f] = off ? off[f] : -1;
}

// The library's nodal projection on the host.  Geometry: dm, n[3], dx[3], per/dlo/dhi flags;
// arrays as mac_hgproject_dense.  phi_out (nullable) receives the nodal solution.  stats_out:
// [status, cycles, rel_resid, fnorm].
// inner > 0: the mixed-precision solve with `inner` FP32 V-cycles per FP64 refinement step.
int hgh_project_prec(int dm, const int* n, const double* dx, const int* per, const int* dlo,
                     const int* dhi, int dense, int proj_type, double dt, int alt, double rel_eps,
                     int max_cycles, int nu1, int nu2, int inner, double* unew,
                     const double* uold, double* gpi, const double* rhohalf, double* pi,
                     const double* b0, const double* nodalrhs, double* phi_out,
                     double* stats_out) {
    hg::Geo G{};
    G.dm = dm;
    for (int d = 0; d < 3; ++d) {
        G.per[d] = d < dm ? per[d] : 0;
        G.dlo[d] = d < dm ? dlo[d] : 0;
        G.dhi[d] = d < dm ? dhi[d] : 0;
    }
    G.dense = dense;
    bool dir = false;
    for (int d = 0; d < dm; ++d) dir = dir || G.dlo[d] || G.dhi[d];
    std::vector<hg::LevT<double>> shape;
    int nn[3];
    double h[3];
    for (int d = 0; d < 3; ++d) {
        nn[d] = d < dm ? n[d] : 1;
        h[d] = d < dm ? dx[d] : 1.0;
    }
    while (true) {
        hg::LevT<double> S{};
        for (int d = 0; d < 3; ++d) {
            S.n[d] = nn[d];
            S.nn[d] = d < dm ? nn[d] + 1 : 1;
            S.h[d] = h[d];
        }
        shape.push_back(S);
        bool more = (int)shape.size() < hg::kMaxLevels;
        for (int d = 0; d < dm; ++d) more = more && nn[d] % 2 == 0 && nn[d] >= 4;
        if (!more) break;
        for (int d = 0; d < dm; ++d) {
            nn[d] /= 2;
            h[d] *= 2;
        }
    }
    HostExec E;
    E.build(G, !dir, shape);
    HostMg<float> E32;
    E32.build(G, !dir, shape);
    E.v32 = &E32;
    E.proj_type = proj_type;
    E.dt = dt;
    E.unew = unew;
    E.uold = uold;
    E.gpi = gpi;
    E.rhohalf = rhohalf;
    E.pi = pi;
    E.b0 = b0;
    E.nodalrhs = nodalrhs;
    E.wall = g_wall;
    E.alt = (proj_type != hg::kInitial && proj_type != hg::kDivuIters && alt) ? 1 : 0;
    hg::SolveStats S{};
    const int rc = inner > 0
                       ? hg::project_mixed(E, E32, rel_eps, max_cycles, nu1, nu2, inner, &S)
                       : hg::project(E, rel_eps, max_cycles, nu1, nu2, &S);
    if (phi_out) std::copy(E.store[hg::kPhi][0].begin(), E.store[hg::kPhi][0].end(), phi_out);
    if (stats_out) {
        stats_out[0] = rc;
        stats_out[1] = S.cycles;
        stats_out[2] = S.rel_resid;
        stats_out[3] = S.fnorm;
    }
    return rc;
}

int hgh_project(int dm, const int* n, const double* dx, const int* per, const int* dlo,
                const int* dhi, int dense, int proj_type, double dt, int alt, double rel_eps,
                int max_cycles, int nu1, int nu2, double* unew, const double* uold, double* gpi,
                const double* rhohalf, double* pi, const double* b0, const double* nodalrhs,
                double* phi_out, double* stats_out) {
    return hgh_project_prec(dm, n, dx, per, dlo, dhi, dense, proj_type, dt, alt, rel_eps,
                            max_cycles, nu1, nu2, 0, unew, uold, gpi, rhohalf, pi, b0, nodalrhs,
                            phi_out, stats_out);
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

// node_row against node_op on one level: random sigma and phi, every node; returns the largest
// |sum_m w_m phi_m - (diag phi_p - off)| relative to max |diag phi_p - off| (0 when they agree).
double hgh_row_check(int dm, const int* n, const double* dx, const int* per, const int* dlo,
                     const int* dhi, int dense, unsigned seed) {
    mac::hg::Geo G{};
    G.dm = dm;
    G.dense = dense;
    for (int d = 0; d < 3; ++d) {
        G.per[d] = d < dm ? per[d] : 0;
        G.dlo[d] = d < dm ? dlo[d] : 0;
        G.dhi[d] = d < dm ? dhi[d] : 0;
    }
    mac::hg::Lev L{};
    for (int d = 0; d < 3; ++d) {
        L.n[d] = d < dm ? n[d] : 1;
        L.nn[d] = d < dm ? n[d] + 1 : 1;
        L.h[d] = d < dm ? dx[d] : 1.0;
    }
    mac::hg::set_dense_weights(dm, L);
    const long nc = mac::hg::ncells(L), nn = mac::hg::nnodes(L);
    std::vector<double> sig(nc), phi(nn);
    unsigned st = seed ? seed : 1u;
    auto rnd = [&]() {
        st = st * 1664525u + 1013904223u;
        return (double)(st >> 8) / 16777216.0;
    };
    for (auto& v : sig) v = 0.5 + rnd();
    for (auto& v : phi) v = rnd() - 0.5;
    L.sig = sig.data();
    double worst = 0.0, scale = 0.0;
    for (long idx = 0; idx < nn; ++idx) {
        int p[3];
        mac::hg::node_coords(L, idx, p);
        double dg, off;
        mac::hg::node_op(G, L, p, phi.data(), dg, off);
        const double ref = dg * phi[idx] - off;
        double sum = 0.0;
        mac::hg::node_row(G, L, p, [&](long m, double w) { sum += w * phi[m]; });
        worst = std::max(worst, std::fabs(sum - ref));
        scale = std::max(scale, std::fabs(ref));
    }
    return scale > 0.0 ? worst / scale : worst;
}

}  // extern "C"
