/*
 * maestro_mac.h -- C ABI of the GB300 (sm_103a) MAC projection.
 *
 * Drop-in for MAESTRO's MAC projection hot path:
 *   subroutine macproject(mla, umac, phi, rho, dx, the_bc_tower,
 *                         macrhs, beta0_1d, beta0_1d_edge, beta0_cart_edge)
 *       Source/macproject.f90:51-76
 *   subroutine mac_multigrid(mla, rh, phi, fine_flx, solver_alpha, solver_beta, dx,
 *                            the_bc_tower, bc_comp, stencil_order,
 *                            rel_solver_eps, abs_solver_eps)
 *       Source/mac_multigrid.f90:18-37 (forwards to FBoxLib ml_cc_solve, :56-67)
 *   subroutine cell_to_edge(s0_cell, s0_edge)
 *       Source/cell_to_edge.f90:14
 *
 * Plain pointers and sizes only.  Every entry point returns MAC_OK (0) or a negative MAC_ERR_*
 * code (the reference aborts through bl_error instead, Source/macproject.f90:99-109).
 * A context is single-threaded: one host thread and one CUDA stream at a time.
 *
 * Data layout at the boundary is FBoxLib's: one Fortran-ordered fab per box, indexed
 * (lo-ng : hi+ng) per direction, edge (face) fabs one longer in their own direction, cell
 * multi-component fabs (..., ncomp).  Box bounds are 0-based inclusive cell indices (lwb/upb).
 * In 2-D the vertical direction is y, in 3-D it is z (MAESTRO planar geometry).
 */
#ifndef MAESTRO_MAC_H
#define MAESTRO_MAC_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------ */
#define MAC_OK                 0
#define MAC_ERR_INVALID       -1   /* bad argument: sizes, boxes, BCs, null pointers          */
#define MAC_ERR_CUDA          -2   /* a CUDA runtime call failed                               */
#define MAC_ERR_NOT_CONVERGED -3   /* max_vcycles reached above the tolerance                  */
#define MAC_ERR_NONFINITE     -4   /* NaN/Inf met in the right-hand side or the residual       */
#define MAC_ERR_ALLOC         -5   /* device memory allocation failed                          */
#define MAC_ERR_UNSUPPORTED   -6   /* geometry the solver does not handle (see mac_strerror)   */
#define MAC_ERR_BAD_DENSITY   -7   /* rho <= 0 or non-finite (face coefficients undefined)     */
#define MAC_ERR_TOO_LARGE     -8   /* size above a fixed limit of the entry point              */
#define MAC_ERR_DEVICE_TIMEOUT -9  /* a kernel's bounded wait for its own async copies expired  */

/* ---- boundary codes: FBoxLib bc_module numbering of ell_bc_level_array(...,press_comp) ---- */
#define MAC_BC_PER  -1   /* periodic                                       */
#define MAC_BC_INT   0   /* interior (not a domain boundary; rejected here) */
#define MAC_BC_DIR   1   /* homogeneous Dirichlet on phi (outlet)          */
#define MAC_BC_NEU   2   /* homogeneous Neumann on phi (walls, inlet, symmetry) */

/* ---- precision of the solve ---------------------------------------------------------------- */
#define MAC_PREC_FP64   0   /* FP64 V-cycles: the plain drop-in                                */
#define MAC_PREC_MIXED  1   /* FP32 V-cycles inside FP64 iterative refinement                  */

/* ---- where the caller's pointers live ------------------------------------------------------ */
#define MAC_PTR_HOST    0
#define MAC_PTR_DEVICE  1

typedef struct mac_ctx mac_ctx;

/* Single-level geometry: the domain, its cell size, the elliptic BCs of press_comp and the boxes
 * of the layout (ml_layout / boxarray of the one level). */
typedef struct mac_geom {
    int dm;                 /* 2 or 3                                                          */
    int domain_lo[3];       /* problem domain, inclusive cell indices (entries >= dm ignored)  */
    int domain_hi[3];
    double dx[3];           /* cell size per direction                                         */
    int bc_lo[3];           /* MAC_BC_* on the low side of each direction                       */
    int bc_hi[3];           /* MAC_BC_* on the high side                                        */
    int nboxes;
    const int* box_lo;      /* [nboxes*3] inclusive lower cell index of each box (x fastest)   */
    const int* box_hi;      /* [nboxes*3] inclusive upper cell index                            */
} mac_geom;

/* Solver options; mac_default_opts() fills MAESTRO's MAC settings. */
typedef struct mac_opts {
    int precision;          /* MAC_PREC_FP64 / MAC_PREC_MIXED                                  */
    int use_alt_energy_fix; /* solver coefficient beta0^2/rho instead of beta0/rho
                               (Source/macproject.f90:189-192; probin default .true.)          */
    double rel_eps;         /* relative tolerance on ||f - L phi||_inf / ||f||_inf;
                               default min(eps_mac * 10^(nlevs-1), eps_mac_max) = 1e-10
                               (Source/macproject.f90:217, Source/mg_eps.f90:23-28)            */
    double abs_eps;         /* absolute tolerance (<= 0: off; the reference passes -1)         */
    int max_vcycles;        /* V-cycles (FP64) or refinement iterations (mixed) before
                               MAC_ERR_NOT_CONVERGED                                           */
    int nu1, nu2;           /* GS-RB sweeps down / up the V-cycle (FBoxLib defaults 2, 2)      */
    int nub;                /* sweeps before and after the bottom solve (mg_bottom_nu = 10)    */
    double bottom_eps;      /* bottom BiCGStab relative tolerance (eps_mac_bottom = 1e-3)      */
    int bottom_max_iter;    /* bottom BiCGStab iteration limit                                 */
    int max_levels;         /* 0: coarsen every box down to 2 cells per side (FBoxLib rule);
                               > 0: cap on the number of MG levels                             */
    int use_graph;          /* capture each V-cycle in a CUDA graph (1) or launch directly (0) */
    int verbose;            /* 0 silent, 1 per-solve summary on stderr                         */
    int timing;             /* 1: CUDA-event timing of the finest-level kernel classes into
                               mac_stats.ktime_* (events recorded inside the V-cycle graph)    */
    int inner_vcycles;      /* mixed precision: FP32 V-cycles per FP64 refinement step (>= 1;
                               default 3; the most per step when adaptive_inner is on); the
                               FP64 residual is formed once per step                          */
    int coarse_tail;        /* 1 (default): the levels small enough for shared memory and the
                               bottom solve run as one single-CTA kernel (same arithmetic)     */
    int adaptive_inner;     /* mixed precision, 1 (default): after each step the next step runs
                               only as many inner V-cycles (<= inner_vcycles) as the contraction
                               just observed predicts the tolerance needs; 0: always
                               inner_vcycles                                                   */
    int inner_krylov;       /* mixed precision with inner_nu2 > 0 and inner_omega = 1: 1 = the
                               inner FP32 V-cycles of a step precondition a flexible
                               conjugate-gradient iteration (one previous direction kept; each
                               V-cycle starts from zero on the current FP32 residual): fewer
                               V-cycles, but at the same residual tolerance the projected
                               velocity can be further from the converged one; 0 (default) =
                               the V-cycles applied one after the other                        */
    int inner_nu1, inner_nu2; /* mixed precision: red/black sweeps down / up the inner FP32
                               V-cycles (default 2 / 1; -1: nu1 / nu2); the FP64 V-cycle always
                               uses nu1 / nu2                                                  */
    int inner_exact_bottom; /* mixed precision, 1 (default): the inner V-cycles solve a bottom of
                               at most 64 cells exactly, by its dense FP64 (pseudo-)inverse
                               formed once per solve; 0: FP64 BiCGStab as the FP64 V-cycle     */
    double inner_omega;     /* mixed precision: relaxation weight of the inner V-cycles'
                               red/black half-sweeps, 0 < omega < 2 (default 1.25; 1:
                               Gauss-Seidel)                                                   */
    double wait_limit_s;    /* seconds a kernel waits for its own asynchronous copies before it
                               gives up, records the failure and returns; the call then reports
                               MAC_ERR_DEVICE_TIMEOUT (0 < wait_limit_s <= 10; default 1)      */
    int inject_wait_expiry; /* fault injection for failure-handling tests (default 0): 1 = the
                               first wait of every staged finest-level kernel waits on a barrier
                               that no copy completes, so it expires after wait_limit_s and the
                               call returns MAC_ERR_DEVICE_TIMEOUT; the GPU and the context stay
                               usable                                                          */
    int fused_sweep;        /* mixed precision, 1: each red/black sweep of the finest FP32 level
                               runs as one kernel (one HBM pass, the same arithmetic, bitwise
                               the same result); 0 (default): two half-sweep kernels          */
} mac_opts;

/* Kernel classes of mac_stats.ktime_* (finest level unless stated). */
#define MAC_KT_SMOOTH    0   /* red/black half sweeps (Gauss-Seidel or over-relaxed)          */
#define MAC_KT_RESTRICT  1   /* defect + restriction to level 1                               */
#define MAC_KT_COARSE    2   /* everything on levels >= 1 incl. the bottom solve              */
#define MAC_KT_PROLONG   3   /* prolongation from level 1                                     */
#define MAC_KT_ACCUM     4   /* FP64 accumulation phi += e and the inner Krylov steps (mixed) */
#define MAC_KT_RESID     5   /* convergence residual (FP64)                                   */
#define MAC_KT_SETUP     6   /* coefficients, right-hand side, layout conversion              */
#define MAC_KT_CORRECT   7   /* velocity correction + layout conversion                       */
#define MAC_KT_NCLASS    8

typedef struct mac_stats {
    int status;             /* return code of the call                                         */
    int vcycles;            /* V-cycles run (mixed: FP32 V-cycles summed over the steps)       */
    int refine_iters;       /* FP64 refinement iterations (mixed precision), else 0            */
    int nlevels;            /* MG levels used                                                  */
    int bottom_iters;       /* BiCGStab iterations summed over the solve                        */
    double fnorm;           /* ||f||_inf of the solver right-hand side (after mean removal)    */
    double resid0;          /* initial ||f - L phi||_inf                                       */
    double rel_resid;       /* final ||f - L phi||_inf / ||f||_inf, FP64                       */
    int nhist;
    double hist[64];        /* relative residual after every V-cycle / refinement iteration    */
    double setup_ms;        /* device time: layout conversion + coefficients + RHS             */
    double solve_ms;        /* device time: multigrid                                          */
    double total_ms;        /* wall time of the call                                           */
    long long launches;     /* CUDA kernels this call launched (graph replays included)         */
    double ktime_ms[8];     /* device time per MAC_KT_* class (opts.timing), summed            */
    int ktime_launches[8];  /* kernel launches per class                                       */
} mac_stats;

/* Fill *o with MAESTRO's MAC-projection defaults (FP64, alt energy fix off, 1e-10, V(2,2),
 * nub = 10, bottom 1e-3). */
void mac_default_opts(mac_opts* o);

/* Human-readable text of a status code (static storage). */
const char* mac_strerror(int code);

/* Library version string (static storage). */
const char* mac_version(void);

/* Create a solver context for one level geometry; device buffers are allocated here and reused
 * by every call.  `cuda_stream` is a cudaStream_t (NULL: the legacy default stream). */
int mac_ctx_create(mac_ctx** out, const mac_geom* g, const mac_opts* o, void* cuda_stream);
int mac_ctx_destroy(mac_ctx* ctx);
/* Replace the options of an existing context (precision, tolerances, sweeps). */
int mac_ctx_set_opts(mac_ctx* ctx, const mac_opts* o);
/* Number of MG levels and the cell counts of each (n[3*l + d]); returns the level count. */
int mac_ctx_levels(const mac_ctx* ctx, int* n_out /* [3*32] or NULL */);

/*
 * MAC projection, the drop-in for macproject (Source/macproject.f90:51-328), single level,
 * planar (beta0_1d) or no-beta0 form.
 *   umac[d*nboxes + b] : edge fab of box b normal to direction d, ng_u ghosts   (in/out)
 *   phi[b]             : cell fab, ng_phi ghosts; initial guess in, solution out (in/out)
 *   rho[b]             : cell state fab with rho_ncomp components, ng_rho ghosts; component
 *                        rho_comp (0-based) is the density (rho_comp in Source/variables.f90:105)
 *   macrhs[b]          : cell fab, ng_rhs ghosts, or NULL (no source term)
 *   beta0_1d           : nr = domain extent in the vertical direction, or NULL
 *   beta0_1d_edge      : nr + 1 edge values, NULL iff beta0_1d is NULL
 * `ptr_kind` says whether all of these live in host or device memory.  On return the valid
 * faces of umac hold the projected velocity; same-level and periodic ghost faces are refilled
 * from the valid region (multifab_fill_boundary, Source/macproject.f90:245-251); physical-
 * boundary ghosts are left to the caller (multifab_physbc_edgevel).
 */
int mac_macproject(mac_ctx* ctx, int ptr_kind,
                   double* const* umac, int ng_u,
                   double* const* phi, int ng_phi,
                   const double* const* rho, int ng_rho, int rho_ncomp, int rho_comp,
                   const double* const* macrhs, int ng_rhs,
                   const double* beta0_1d, const double* beta0_1d_edge,
                   mac_stats* stats);

/*
 * Elliptic solve, the drop-in for mac_multigrid (Source/mac_multigrid.f90:18-67):
 *   (alpha - div beta grad) phi = rh
 * with face coefficients beta[d*nboxes + b] (edge fabs, ng_beta ghosts) and optional cell
 * alpha[b] (NULL: alpha = 0, the MAC case).  phi is the initial guess in / solution out.
 * fine_flx is not returned: on one level the face flux beta grad phi is formed by the caller
 * from phi (mac_macproject does so internally).
 */
int mac_multigrid(mac_ctx* ctx, int ptr_kind,
                  const double* const* rh, int ng_rh,
                  double* const* phi, int ng_phi,
                  const double* const* alpha, int ng_alpha,
                  const double* const* beta, int ng_beta,
                  mac_stats* stats);

/*
 * Whole-domain variant of mac_macproject for callers that keep one array per field on the
 * device (natural layout, x fastest, no ghosts): ux (nx+1,ny,nz), uy (nx,ny+1,nz),
 * uz (nx,ny,nz+1) (uz unused in 2-D), phi/rho/macrhs (nx,ny,nz), beta0 (nr), beta0_edge (nr+1).
 * All pointers are device pointers; macrhs/beta0/beta0_edge may be NULL as above.
 * Same arithmetic as mac_macproject.  No counterpart in the reference (its fields always come
 * boxed); it is the device-resident form of Source/macproject.f90:51-328.
 */
int mac_macproject_dense(mac_ctx* ctx, double* ux, double* uy, double* uz, double* phi,
                         const double* rho, const double* macrhs, const double* beta0,
                         const double* beta0_edge, mac_stats* stats);

/*
 * MAC projection in the spherical form: beta0 given on every face (the beta0_cart_edge
 * multifab argument of macproject, Source/macproject.f90:79, 103-109, 155-161, 194-201,
 * 236-241), as MAESTRO's spherical geometry calls it on its Cartesian grid.  Arguments as
 * mac_macproject with beta0_1d / beta0_1d_edge replaced by
 *   beta0_cart_edge[d*nboxes + b] : edge fab of box b normal to direction d, ng_b ghosts (in)
 * All fabs live where `ptr_kind` says.  U *= beta0 face by face, solver beta = beta0^p 2 /
 * (rho_L + rho_R) (p = 1, 2 with use_alt_energy_fix), U = (beta0 U - beta grad phi) / beta0.
 */
int mac_macproject_cart(mac_ctx* ctx, int ptr_kind,
                        double* const* umac, int ng_u,
                        double* const* phi, int ng_phi,
                        const double* const* rho, int ng_rho, int rho_ncomp, int rho_comp,
                        const double* const* macrhs, int ng_rhs,
                        const double* const* beta0_cart_edge, int ng_b,
                        mac_stats* stats);

/*
 * Whole-domain device-array variant of mac_macproject_cart (natural layout as in
 * mac_macproject_dense): b0x (nx+1,ny,nz), b0y (nx,ny+1,nz), b0z (nx,ny,nz+1) the beta0 faces
 * (b0z unused in 2-D); macrhs may be NULL.
 */
int mac_macproject_cart_dense(mac_ctx* ctx, double* ux, double* uy, double* uz, double* phi,
                              const double* rho, const double* macrhs, const double* b0x,
                              const double* b0y, const double* b0z, mac_stats* stats);

/*
 * Multi-level (AMR) hierarchy of a context, replacing the ml_layout `mla` of
 * macproject(mla, umac(nlev,dm), phi(nlev), rho(nlev), dx(nlev,dm), the_bc_tower, macrhs(nlev),
 * beta0_1d(nlev,:), beta0_1d_edge(nlev,:)) (Source/macproject.f90:51-76) for nlevs > 1.
 * Level 0 is the context's own geometry; levels 1 .. nlev-1 refine by 2 and are given by their
 * boxes in level-l cell indices: nboxes[l] boxes for l >= 1 (nboxes[0] is ignored), their lo / hi
 * corners (3 ints each, level 1's boxes first) in box_lo / box_hi.  Every box is aligned to the
 * ratio (even lo, odd hi) and properly nested: its cells coarsened and grown by one cell in every
 * direction lie in the level below (or beyond a non-periodic domain face).  nlev == 1 drops the
 * hierarchy.  Returns MAC_ERR_INVALID for a bad layout.
 */
int mac_ctx_set_amr(mac_ctx* ctx, int nlev, const int* nboxes, const int* box_lo,
                    const int* box_hi);

/*
 * Multi-level MAC projection (Source/macproject.f90:51-328 with nlevs > 1) on whole-level-domain
 * DEVICE arrays, Fortran order: level l spans (n[d] << l) cells along each direction of the
 * context's domain; only the cells of its boxes (and for rho one cell around them) and the faces
 * bordering them are read or written.  umac[3*l + d] faces of level l (n_l[d] + 1 along d; in/out),
 * phi[l] cells (in: initial guess; out: the composite solution, covered cells the mean of their
 * children), rho[l] cells, macrhs (NULL, or per level, entries may be NULL), beta0[l] /
 * beta0_edge[l] the planar base state of level l (n_l[dm-1] and n_l[dm-1] + 1 values; NULL
 * together: no beta0).  The composite problem (coarse-fine ghosts, reflux) is described in the
 * library's mac_amr.cuh; the tolerance is min(rel_eps * 10^(nlev-1), 1e-8) as in MAESTRO
 * (Source/macproject.f90:217).  A context created with MAC_PREC_FP64 runs FP64 multi-level cycles;
 * one created with MAC_PREC_MIXED runs FP32 multi-level cycles under FP64 refinement (FP64
 * composite residual, accumulation and convergence test; the level-0 coarse correction is an
 * FP64 V-cycle).  Needs mac_ctx_set_amr.
 */
int mac_macproject_ml_dense(mac_ctx* ctx, double* const* umac, double* const* phi,
                            const double* const* rho, const double* const* macrhs,
                            const double* const* beta0, const double* const* beta0_edge,
                            mac_stats* stats);

/*
 * Multi-level MAC projection on the caller's boxes, the drop-in for macproject with nlevs > 1
 * (Source/macproject.f90:51-328).  Arguments as mac_macproject, with the fab lists of all levels
 * one after the other (level 0 = the context's boxes, then the boxes of mac_ctx_set_amr in
 * order):
 *   umac   : per level, dm blocks of that level's nboxes edge fabs (direction-major, as in
 *            mac_macproject), ng_u ghosts (in/out: the boxes' own faces are written)
 *   phi    : per level, one cell fab per box, ng_phi ghosts (in: guess; out: the boxes' cells)
 *   rho    : per level, one state fab per box, rho_ncomp components, ng_rho >= 1 ghosts (the
 *            coarse-fine faces read the density one cell outside the level)
 *   macrhs : per level, one cell fab per box, ng_rhs ghosts, or NULL
 *   beta0 / beta0_edge : the levels' planar base states one after the other (n_l and n_l + 1
 *            values, n_l = the level's vertical extent), or both NULL
 * After the projection the fine levels' ghost faces (ng_u >= 1) are filled as create_umac_grown
 * fills them (Source/macproject.f90:264-272): a ghost face bordering a cell of the level (another
 * box, periodic images) takes the level's value, any other the coarser level's -- piecewise
 * constant across the face, linear along its normal.  Ghost faces beyond a non-periodic domain
 * face (multifab_physbc_edgevel), level 0's ghost faces and all ghost cells of phi are left as
 * they came in.  Along a periodic
 * direction a domain face is read from the box that owns it (a box at the low end owns face 0,
 * one at the high end face n_l); where only one end has a box, that copy stands for both.
 */
int mac_macproject_ml(mac_ctx* ctx, int ptr_kind,
                      double* const* umac, int ng_u,
                      double* const* phi, int ng_phi,
                      const double* const* rho, int ng_rho, int rho_ncomp, int rho_comp,
                      const double* const* macrhs, int ng_rhs,
                      const double* beta0, const double* beta0_edge,
                      mac_stats* stats);

/* proj_type values of the nodal projection (Source/proj_parameters.f90) */
#define MAC_HG_INITIAL        1   /* initial projection: U projected, pi = gpi = 0             */
#define MAC_HG_DIVU_ITERS     2   /* divu iterations: as the initial projection                */
#define MAC_HG_PRESSURE_ITERS 3   /* (U - Uold)/dt projected; U = Uold + dt U; pi, gpi += ...   */
#define MAC_HG_REGULAR        4   /* U + dt gpi/rhohalf projected; pi = phi/dt, gpi = gphi/dt  */

/*
 * Nodal (HG) projection on one level, the drop-in for hgproject (Source/hgproject.f90:32-264,
 * solve Source/hg_multigrid.f90:18-239) on whole-domain DEVICE arrays of the context's geometry
 * (Fortran order, no ghosts): unew / uold / gpi cell vector fields (n0, n1[, n2], dm),
 * rhohalf and beta0_cart (NULL: 1) cells, pi and nodalrhs (NULL: none) nodes
 * (n0+1, n1+1[, n2+1]).  proj_type MAC_HG_*, dt the time step (> 0 for the pressure iterations
 * and the regular time step), dense_stencil 1 for hg_dense_stencil (9/27-point) else the cross
 * stencil, rel_eps the solver tolerance (<= 0: eps_hg = 1e-12).  Walls (U.n = 0), periodic and
 * outflow (phi = 0) faces (inlets: mac_ctx_set_inflow, mac_hgproject_dense_inflow); the
 * context's use_alt_energy_fix, max_vcycles, nu1 and nu2 apply.
 * unew, gpi and pi are updated in place.
 */
int mac_hgproject_dense(mac_ctx* ctx, int proj_type, double dt, int dense_stencil, double rel_eps,
                        double* unew, const double* uold, double* gpi, const double* rhohalf,
                        double* pi, const double* beta0_cart, const double* nodalrhs,
                        mac_stats* stats);

/*
 * Nodal (HG) projection on the caller's boxes (the context's layout), the drop-in for hgproject
 * (Source/hgproject.f90:32-264) on one level.  Per box b: unew[b], uold[b] (NULL array unless
 * MAC_HG_PRESSURE_ITERS), gpi[b] cell fabs with dm components; rhohalf[b] and beta0_cart[b]
 * (NULL array: beta0 = 1) cell fabs; pi[b] and nodalrhs[b] (NULL array: none) node fabs (one more
 * entry than the box along every direction); each array with its ghost width.  The boxes' own
 * cells of unew and gpi and their nodes of pi are written; ghosts are left as they came in.
 * Other arguments as mac_hgproject_dense.
 */
int mac_hgproject(mac_ctx* ctx, int ptr_kind, int proj_type, double dt, int dense_stencil,
                  double rel_eps, double* const* unew, int ng_u, const double* const* uold,
                  int ng_uo, double* const* gpi, int ng_gp, const double* const* rhohalf,
                  int ng_rho, double* const* pi, int ng_pi, const double* const* beta0_cart,
                  int ng_b0, const double* const* nodalrhs, int ng_nr, mac_stats* stats);

/*
 * Inflow (inlet) faces of the nodal projection: the phys_bc == INLET test of hg_multigrid
 * (Source/hg_multigrid.f90:191-203).  lo_inflow[d] / hi_inflow[d] (0 or 1; entries >= dm
 * ignored; NULL: none) mark the low / high face of direction d as an inlet, which must be a
 * MAC_BC_NEU face (MAC_ERR_INVALID otherwise).  Until the next call, the node-centred divergence
 * of the nodal entries takes at an inlet the flux through the face of the inflow velocity on the
 * wall: the normal component of U in the ghost cell just outside the face, as hgproject leaves it
 * (create_uvec_for_projection: (U - Uold) / dt for the pressure iterations, else unchanged;
 * times beta0_cart there when beta0_cart has a ghost layer).  Cells outside other non-periodic
 * faces carry U = 0.  mac_hgproject reads the ghost values from the fabs (ng_u >= 1, and
 * ng_uo >= 1 for MAC_HG_PRESSURE_ITERS; MAC_ERR_INVALID otherwise); mac_hgproject_dense_inflow
 * takes them as an array.  The MAC projection needs none of this: its inlet face velocities are
 * part of umac.
 */
int mac_ctx_set_inflow(mac_ctx* ctx, const int* lo_inflow, const int* hi_inflow);

/*
 * mac_hgproject_dense with inflow faces.  inflow_wall (DEVICE): for each inflow face of
 * mac_ctx_set_inflow in the order (d = 0 low, d = 0 high, d = 1 low, ...), the wall value of
 * beta0 U_d (the ghost cell's normal velocity after create_uvec_for_projection and the beta0
 * scaling) for every cell of the face, the face's other directions in Fortran order; NULL exactly
 * when no inflow face is set (MAC_ERR_INVALID otherwise).  mac_hgproject_dense is this entry with
 * inflow_wall NULL.
 */
int mac_hgproject_dense_inflow(mac_ctx* ctx, int proj_type, double dt, int dense_stencil,
                               double rel_eps, double* unew, const double* uold, double* gpi,
                               const double* rhohalf, double* pi, const double* beta0_cart,
                               const double* nodalrhs, const double* inflow_wall,
                               mac_stats* stats);

/*
 * Adjoint (reverse-mode derivative) of the whole-domain MAC projection; no counterpart in the
 * reference.  Forward map (beta0 form, p = 1 + use_alt_energy_fix):
 *   U_proj = U - c .* G phi,  A phi = f,  A = D diag(beta_f) G  (negated, alpha = 0),
 *   beta_f = beta0_f^p * 2/(rho_L + rho_R),  c = beta_f / beta0_f,
 *   f = macrhs - D(beta0_f U).
 * Given the cotangent w = dL/dU_proj (face arrays like U), returns
 *   dU     = dL/dU            (face arrays, natural layout, device)
 *   drinv  = dL/d(1/rho)      (cells, device; may be NULL)
 *   dbeta0 = dL/d(beta0_1d)   (nr cells, device; may be NULL) -- beta0_edge is taken as a
 *            function of beta0 through cell_to_edge, so this includes the edge path
 *   dmacrhs= dL/d(macrhs)     (cells, device; may be NULL)
 * The adjoint solve reuses the forward V-cycle (A is self-adjoint).  U, rho, macrhs, beta0 are
 * the forward inputs (U before projection).  phi_out (may be NULL) receives the forward phi.
 */
int mac_macproject_adjoint_dense(mac_ctx* ctx,
                                 const double* ux, const double* uy, const double* uz,
                                 const double* rho, const double* macrhs,
                                 const double* beta0, const double* beta0_edge,
                                 const double* wx, const double* wy, const double* wz,
                                 double* dux, double* duy, double* duz,
                                 double* drinv, double* dbeta0, double* dmacrhs,
                                 double* phi_out, mac_stats* stats);

/* ---- allocation-free small solve ----------------------------------------------------------- */
#define MAC_NOALLOC_MAX_CELLS 4096   /* largest level mac_solve_small_noalloc accepts (cells)  */

/*
 * (alpha - div beta grad) phi = rh on one small single-box level, allocating no device memory.
 * No counterpart in the reference.
 * For callers that cannot allocate on the GPU -- a host code whose device memory belongs to its
 * own pool allocator, a loop held to a fixed memory budget, or a call site where cudaMalloc is
 * forbidden or too slow.  The caller passes device pointers to its inputs and output (natural
 * layout, x fastest): rh and phi (n[0]*n[1]*n[2]; phi = initial guess in, solution out),
 * beta_x/y/z face coefficients ((n[d]+1) along d; beta_z unused in 2-D), alpha (cells, or NULL
 * for the MAC case).  Same operator and boundary handling as mac_multigrid; solved by the
 * single-CTA BiCGStab of the multigrid's coarsest level, run to
 * ||rh - L phi||_inf <= rel_eps ||rh||_inf (mean of rh removed when the problem is singular)
 * within max_iter iterations (else MAC_ERR_NOT_CONVERGED).
 * Limits: at most MAC_NOALLOC_MAX_CELLS cells (else MAC_ERR_TOO_LARGE).  Its work storage is one
 * fixed array of 14*MAC_NOALLOC_MAX_CELLS doubles that every GPU loading the library holds until
 * the process exits.  All calls share that array and it keeps the last call's contents; calls
 * that overlap on the GPU (other streams or host threads) race -- serialise them.  The first call
 * on a device looks up the array's address with that device current.  Blocks the host until the
 * solve has finished (it reads the result back).
 */
int mac_solve_small_noalloc(int dm, const int* n, const double* dx, const int* bc_lo,
                            const int* bc_hi, const double* rh, double* phi,
                            const double* beta_x, const double* beta_y, const double* beta_z,
                            const double* alpha, double rel_eps, int max_iter,
                            void* cuda_stream, mac_stats* stats);

/* beta0 cell -> edge values (Source/cell_to_edge.f90:14-70), host arrays, one level. */
int mac_cell_to_edge(int nr, const double* s0_cell, double* s0_edge);

/* ---- producers of the projection's inputs (planar geometry) ----------------------------------
 * mac_make_macrhs replaces make_macrhs (Source/make_macrhs.f90:28-107; 2-D :135-178, 3-D
 * :184-240) for one level:
 *   macrhs = beta0(r) (S_cc - Sbar(r) + delta_gamma1_term)             r = vertical index
 *   if dpdt_factor > 0: delta_chi = 0 first when is_predictor; below the base cutoff
 *   (r < base_cutoff_density_coord) delta_chi += dpdt_factor delta_p_term / (dt gamma1bar(r)
 *   p0(r)) and macrhs += beta0(r) delta_chi.
 * Per-box fabs (host or device pointers, one component each); Sbar, beta0, gamma1bar, p0 are the
 * 1-D base state (nr values, same pointer kind).  gamma1bar, p0, delta_p_term and delta_chi may be
 * NULL when dpdt_factor <= 0.  Difference from the reference: ghost cells of macrhs and
 * delta_chi are filled from their valid images (periodic / neighbouring boxes) instead of being
 * left untouched; ghosts outside non-periodic walls are left untouched. */
int mac_make_macrhs(mac_ctx* ctx, int ptr_kind, double* const* macrhs, int ng_rh,
                    const double* const* S_cc, int ng_sr, const double* const* delta_gamma1_term,
                    int ng_dg, const double* Sbar, const double* beta0, const double* gamma1bar,
                    const double* p0, const double* const* delta_p_term, int ng_dp,
                    double* const* delta_chi, int ng_d, double dt, double dpdt_factor,
                    int base_cutoff_density_coord, int is_predictor);

/* Whole-domain device form of mac_make_macrhs (natural layout (nx,ny[,nz]) arrays, device 1-D
 * base state); no reference counterpart (device-resident drivers). */
int mac_make_macrhs_dense(mac_ctx* ctx, double* macrhs, const double* S_cc,
                          const double* delta_gamma1_term, const double* Sbar,
                          const double* beta0, const double* gamma1bar, const double* p0,
                          const double* delta_p_term, double* delta_chi, double dt,
                          double dpdt_factor, int base_cutoff_density_coord, int is_predictor);

/* mac_make_at_halftime replaces make_at_halftime (Source/make_at_halftime.f90:82-130) for one
 * level: half(out_comp) = (sold(in_comp) + snew(in_comp)) / 2 on valid cells; ghost cells are
 * filled from their valid images (the reference's ml_restrict_and_fill).  half fabs have one
 * component (half_ncomp = 1, out_comp = 0); sold/snew have s_ncomp components. */
int mac_make_at_halftime(mac_ctx* ctx, int ptr_kind, double* const* half, int ng_half,
                         int out_comp, int half_ncomp, const double* const* sold, int ng_old,
                         const double* const* snew, int ng_new, int in_comp, int s_ncomp);

#ifdef __cplusplus
}
#endif
#endif /* MAESTRO_MAC_H */
