// Shared types of the MAC-projection oracle (TEST INFRASTRUCTURE ONLY): the C option and
// statistics structs of the ctypes front end, the single-level MG hierarchy and the index
// helpers used by both the one-level solve (mac_oracle.cpp) and the multi-level composite
// solve (mac_oracle_ml.cpp).
#pragma once

#include <cstddef>
#include <vector>

extern "C" {

// Boundary codes: the FBoxLib bc_module numbering that ell_bc_level_array holds.
enum { ORC_BC_PER = -1, ORC_BC_INT = 0, ORC_BC_DIR = 1, ORC_BC_NEU = 2 };

typedef struct orc_opts {
    int dm;              // 2 or 3
    int n[3];            // cells per direction (n[2] = 1 when dm == 2)
    double dx[3];
    int bc_lo[3];        // ORC_BC_* per direction, low side
    int bc_hi[3];
    int nlevels;         // number of MG levels (>= 1)
    double rel_eps;
    double abs_eps;      // <= 0: unused
    int max_vcycles;
    int nu1, nu2, nub;
    double bottom_eps;
    int bottom_max_iter;
    int alt_energy_fix;  // beta0^2 instead of beta0 in the solver coefficient
    int nthreads;        // <= 0: OpenMP default
} orc_opts;

typedef struct orc_stats {
    int status;          // 0 converged, 1 not converged
    int vcycles;
    double fnorm;        // ||f||_inf after mean removal
    double resid0;       // initial ||f - L phi||_inf
    double rel_resid;    // final ||f - L phi||_inf / ||f||_inf
    int nhist;
    double hist[64];     // relative residual after each V-cycle
    int bottom_iters;    // BiCGStab iterations summed over the solve
} orc_stats;

}  // extern "C"

namespace orc {

using std::size_t;

struct Level {
    int n[3];
    double h[3];
    int act[3];                 // direction carries a stencil arm
    std::vector<double> b[3];   // face coefficient beta_f, natural face layout (n[d]+1 along d)
    std::vector<double> alpha;  // cell alpha (empty -> 0)
    std::vector<double> diag;
    std::vector<double> phi, f, r;
    size_t ncell() const { return (size_t)n[0] * n[1] * n[2]; }
};

struct Ctx {
    orc_opts o;
    std::vector<Level> lev;
    bool singular = false;
    int bottom_iters = 0;
};

inline size_t cidx(const int* n, int i, int j, int k) {
    return (size_t)i + (size_t)n[0] * ((size_t)j + (size_t)n[1] * k);
}
inline size_t fidx(const int* n, int d, int i, int j, int k) {
    const size_t m0 = (size_t)n[0] + (d == 0), m1 = (size_t)n[1] + (d == 1);
    return (size_t)i + m0 * ((size_t)j + m1 * k);
}

// Neighbour of cell index c along d, side s (-1 low, +1 high).  Returns -1 when the face is
// a domain boundary that is not periodic.
inline int nb_index(int c, int s, int nd, int bclo, int bchi) {
    int q = c + s;
    if (q < 0) return bclo == ORC_BC_PER ? nd - 1 : -1;
    if (q >= nd) return bchi == ORC_BC_PER ? 0 : -1;
    return q;
}

void build_diag(Ctx& C, Level& L);
void apply_op(const Ctx& C, const Level& L, const double* u, double* out);
double residual(const Ctx& C, const Level& L, const double* u, const double* f, double* r);
void gsrb(const Ctx& C, Level& L);
double mean_of(const std::vector<double>& v);
void sub_mean(std::vector<double>& v);
double norm_inf(const std::vector<double>& v);
void vcycle(Ctx& C, int l);
void build_hierarchy(Ctx& C, const double* const b[3], const double* alpha);
void set_threads(const orc_opts* o);

}  // namespace orc

extern "C" void orc_mac_coeffs(const orc_opts* o, const double* rho, const double* beta0,
                               const double* beta0_edge, double* bx, double* by, double* bz);
