"""CPU oracle of the MAC projection -- TEST INFRASTRUCTURE ONLY.

ctypes front end of ``mac_oracle.cpp``: an IEEE-FP64 C++/OpenMP restatement of MAESTRO's
``macproject`` (Source/macproject.f90:51-328) and of the FBoxLib cell-centred multigrid that
``mac_multigrid`` (Source/mac_multigrid.f90:18-67) calls.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use this module, and only
as the checker / the timed CPU reference.  The product library never imports it.

Parity status: the reference (Fortran + the un-vendored FBoxLib) cannot be compiled here, so the
oracle is pinned by (a) an MG-independent sparse direct solve of the same discrete system
(scipy, tests/golden/make_golden.py) and (b) the known-answer behaviour of MAESTRO's own
``test_projection`` unit test (Exec/UNIT_TESTS/test_projection/test_projection.f90:172-344,
860-1050): a divergence-free field plus a discrete gradient projects back to the field.  No
numeric golden outputs of the reference exist in its tree, so numerically the parity with the
Fortran code itself is unpinned beyond those two anchors.

Arrays are numpy float64 in Fortran order, indexed like the reference: cell arrays (nx, ny[, nz]),
face arrays with one extra entry along their own direction.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libmac_oracle.so")

# FBoxLib bc_module numbering, as stored in ell_bc_level_array(..., press_comp).
BC_PER, BC_INT, BC_DIR, BC_NEU = -1, 0, 1, 2

# Source/mg_eps.f90:23-28
EPS_MAC, EPS_MAC_MAX, MAC_LEVEL_FACTOR, EPS_MAC_BOTTOM = 1e-10, 1e-8, 10.0, 1e-3


class OrcOpts(ctypes.Structure):
    _fields_ = [
        ("dm", ctypes.c_int),
        ("n", ctypes.c_int * 3),
        ("dx", ctypes.c_double * 3),
        ("bc_lo", ctypes.c_int * 3),
        ("bc_hi", ctypes.c_int * 3),
        ("nlevels", ctypes.c_int),
        ("rel_eps", ctypes.c_double),
        ("abs_eps", ctypes.c_double),
        ("max_vcycles", ctypes.c_int),
        ("nu1", ctypes.c_int),
        ("nu2", ctypes.c_int),
        ("nub", ctypes.c_int),
        ("bottom_eps", ctypes.c_double),
        ("bottom_max_iter", ctypes.c_int),
        ("alt_energy_fix", ctypes.c_int),
        ("nthreads", ctypes.c_int),
    ]


class OrcStats(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int),
        ("vcycles", ctypes.c_int),
        ("fnorm", ctypes.c_double),
        ("resid0", ctypes.c_double),
        ("rel_resid", ctypes.c_double),
        ("nhist", ctypes.c_int),
        ("hist", ctypes.c_double * 64),
        ("bottom_iters", ctypes.c_int),
    ]

    def as_dict(self):
        return {
            "status": self.status,
            "vcycles": self.vcycles,
            "fnorm": self.fnorm,
            "resid0": self.resid0,
            "rel_resid": self.rel_resid,
            "hist": [self.hist[i] for i in range(self.nhist)],
            "bottom_iters": self.bottom_iters,
        }


class OrcHgOpts(ctypes.Structure):
    _fields_ = [
        ("dm", ctypes.c_int),
        ("n", ctypes.c_int * 3),
        ("dx", ctypes.c_double * 3),
        ("bc_lo", ctypes.c_int * 3),
        ("bc_hi", ctypes.c_int * 3),
        ("dense", ctypes.c_int),
        ("proj_type", ctypes.c_int),
        ("dt", ctypes.c_double),
        ("alt_energy_fix", ctypes.c_int),
        ("rel_eps", ctypes.c_double),
        ("max_vcycles", ctypes.c_int),
        ("nu1", ctypes.c_int),
        ("nu2", ctypes.c_int),
        ("bottom_eps", ctypes.c_double),
        ("nthreads", ctypes.c_int),
        ("wall_off", ctypes.c_long * 6),
        ("wall", ctypes.c_void_p),
    ]


_lib = None


_SOURCES = ("mac_oracle.cpp", "mac_oracle_ml.cpp", "hg_oracle.cpp", "mac_oracle_core.h")


def build(force: bool = False) -> str:
    """Compile the oracle sources into oracle/_build/libmac_oracle.so (g++ + OpenMP)."""
    if force or not os.path.exists(_LIB_PATH) or any(
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, f)) for f in _SOURCES
    ):
        subprocess.check_call(["make", "-s", "-C", _HERE], stdout=subprocess.DEVNULL)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER
        d = P(ctypes.c_double)
        L.orc_macproject.argtypes = [P(OrcOpts), d, d, d, d, d, d, d, d, P(OrcStats)]
        L.orc_macproject.restype = ctypes.c_int
        L.orc_macproject_cart.argtypes = [P(OrcOpts), d, d, d, d, d, d, d, d, d, P(OrcStats)]
        L.orc_macproject_cart.restype = ctypes.c_int
        L.orc_mac_multigrid.argtypes = [P(OrcOpts), d, d, d, d, d, d, P(OrcStats)]
        L.orc_mac_multigrid.restype = ctypes.c_int
        L.orc_apply_op.argtypes = [P(OrcOpts), d, d, d, d, d, d]
        L.orc_apply_op.restype = None
        L.orc_mac_coeffs.argtypes = [P(OrcOpts), d, d, d, d, d, d]
        L.orc_mac_coeffs.restype = None
        L.orc_cell_to_edge.argtypes = [ctypes.c_int, d, d]
        L.orc_cell_to_edge.restype = None
        pd = P(d)
        ip = P(ctypes.c_int)
        L.orc_ml_solve.argtypes = [P(OrcOpts), ctypes.c_int, ip, ip, pd, pd, pd, P(OrcStats)]
        L.orc_ml_solve.restype = ctypes.c_int
        L.orc_ml_residual.argtypes = [P(OrcOpts), ctypes.c_int, ip, ip, pd, pd, pd, pd]
        L.orc_ml_residual.restype = ctypes.c_double
        L.orc_macproject_ml.argtypes = [P(OrcOpts), ctypes.c_int, ip, ip, pd, pd, pd, pd, pd, pd,
                                        P(OrcStats)]
        L.orc_macproject_ml.restype = ctypes.c_int
        L.orc_hg_apply.argtypes = [P(OrcHgOpts), d, d, d]
        L.orc_hg_apply.restype = None
        L.orc_hg_divu.argtypes = [P(OrcHgOpts), d, d]
        L.orc_hg_divu.restype = None
        L.orc_hg_grad.argtypes = [P(OrcHgOpts), d, d]
        L.orc_hg_grad.restype = None
        L.orc_hg_solve.argtypes = [P(OrcHgOpts), d, d, d, P(OrcStats)]
        L.orc_hg_solve.restype = ctypes.c_int
        L.orc_hgproject.argtypes = [P(OrcHgOpts), d, d, d, d, d, d, d, d, P(OrcStats)]
        L.orc_hgproject.restype = ctypes.c_int
        L.orc_max_threads.argtypes = []
        L.orc_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def max_threads() -> int:
    return int(lib().orc_max_threads())


def nlevels_for_boxes(box_extents, min_width: int = 2) -> int:
    """MG depth when every box is coarsened by 2 down to `min_width` cells per side.

    FBoxLib coarsens each box of the level while all of its extents stay even and at least
    `min_width` after halving (Docs/mg/mg.tex:227-236: "coarsened as much as they can, down to
    2^3 zones").  `box_extents` is an iterable of per-box extent tuples (cells per direction).
    """
    c = None
    for ext in box_extents:
        for e in ext:
            k = 0
            while e % 2 == 0 and e // 2 >= min_width:
                e //= 2
                k += 1
            c = k if c is None else min(c, k)
    return 1 + (c or 0)


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim == 1)
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _opts(shape, dx, bc_lo, bc_hi, nlevels, rel_eps, abs_eps, max_vcycles, nu1, nu2, nub,
          bottom_eps, bottom_max_iter, alt_energy_fix, threads):
    dm = len(shape)
    o = OrcOpts()
    o.dm = dm
    n = list(shape) + [1] * (3 - dm)
    for d in range(3):
        o.n[d] = int(n[d])
        o.dx[d] = float(dx[d]) if d < dm else 1.0
        o.bc_lo[d] = int(bc_lo[d]) if d < dm else BC_NEU
        o.bc_hi[d] = int(bc_hi[d]) if d < dm else BC_NEU
    o.nlevels = int(nlevels)
    o.rel_eps = rel_eps
    o.abs_eps = abs_eps
    o.max_vcycles = max_vcycles
    o.nu1, o.nu2, o.nub = nu1, nu2, nub
    o.bottom_eps = bottom_eps
    o.bottom_max_iter = bottom_max_iter
    o.alt_energy_fix = int(bool(alt_energy_fix))
    o.nthreads = int(threads)
    return o


def _f64f(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def macproject(umac, phi, rho, dx, bc_lo, bc_hi, macrhs=None, beta0=None, beta0_edge=None,
               nlevels=None, rel_eps=EPS_MAC, abs_eps=-1.0, max_vcycles=100, nu1=2, nu2=2,
               nub=10, bottom_eps=EPS_MAC_BOTTOM, bottom_max_iter=200, alt_energy_fix=False,
               threads=0):
    """Oracle MAC projection on the whole domain.  Returns (umac_new, phi_new, stats)."""
    phi = _f64f(phi).copy(order="F")
    rho = _f64f(rho)
    shape = phi.shape
    dm = len(shape)
    u = [_f64f(x).copy(order="F") for x in umac]
    for d in range(dm):
        exp = list(shape)
        exp[d] += 1
        assert u[d].shape == tuple(exp), (d, u[d].shape, exp)
    if nlevels is None:
        nlevels = nlevels_for_boxes([shape])
    o = _opts(shape, dx, bc_lo, bc_hi, nlevels, rel_eps, abs_eps, max_vcycles, nu1, nu2, nub,
              bottom_eps, bottom_max_iter, alt_energy_fix, threads)
    st = OrcStats()
    rhs = _f64f(macrhs) if macrhs is not None else None
    b0 = np.ascontiguousarray(beta0, dtype=np.float64) if beta0 is not None else None
    b0e = np.ascontiguousarray(beta0_edge, dtype=np.float64) if beta0_edge is not None else None
    uz = u[2] if dm == 3 else None
    lib().orc_macproject(ctypes.byref(o), _ptr(u[0]), _ptr(u[1]), _ptr(uz), _ptr(phi), _ptr(rho),
                         _ptr(rhs), _ptr(b0), _ptr(b0e), ctypes.byref(st))
    return u, phi, st.as_dict()


def macproject_cart(umac, phi, rho, dx, bc_lo, bc_hi, beta0_cart_edge, macrhs=None,
                    nlevels=None, rel_eps=EPS_MAC, abs_eps=-1.0, max_vcycles=100, nu1=2, nu2=2,
                    nub=10, bottom_eps=EPS_MAC_BOTTOM, bottom_max_iter=200,
                    alt_energy_fix=False, threads=0):
    """Oracle MAC projection with beta0 given on every face (the spherical form,
    beta0_cart_edge: one face array per direction, n[d]+1 faces along d).  Returns
    (umac_new, phi_new, stats)."""
    phi = _f64f(phi).copy(order="F")
    rho = _f64f(rho)
    shape = phi.shape
    dm = len(shape)
    u = [_f64f(x).copy(order="F") for x in umac]
    b = [_f64f(x) for x in beta0_cart_edge]
    for d in range(dm):
        exp = list(shape)
        exp[d] += 1
        assert u[d].shape == tuple(exp) and b[d].shape == tuple(exp), (d, u[d].shape, exp)
    if nlevels is None:
        nlevels = nlevels_for_boxes([shape])
    o = _opts(shape, dx, bc_lo, bc_hi, nlevels, rel_eps, abs_eps, max_vcycles, nu1, nu2, nub,
              bottom_eps, bottom_max_iter, alt_energy_fix, threads)
    st = OrcStats()
    rhs = _f64f(macrhs) if macrhs is not None else None
    uz = u[2] if dm == 3 else None
    bz = b[2] if dm == 3 else None
    lib().orc_macproject_cart(ctypes.byref(o), _ptr(u[0]), _ptr(u[1]), _ptr(uz), _ptr(phi),
                              _ptr(rho), _ptr(rhs), _ptr(b[0]), _ptr(b[1]), _ptr(bz),
                              ctypes.byref(st))
    return u, phi, st.as_dict()


def mac_multigrid(rh, phi, beta, dx, bc_lo, bc_hi, alpha=None, nlevels=None, rel_eps=EPS_MAC,
                  abs_eps=-1.0, max_vcycles=100, nu1=2, nu2=2, nub=10,
                  bottom_eps=EPS_MAC_BOTTOM, bottom_max_iter=200, threads=0):
    """Oracle of mac_multigrid: solve (alpha - div beta grad) phi = rh.  Returns (phi, stats)."""
    rh = _f64f(rh)
    phi = _f64f(phi).copy(order="F")
    shape = rh.shape
    dm = len(shape)
    b = [_f64f(x) for x in beta]
    if nlevels is None:
        nlevels = nlevels_for_boxes([shape])
    o = _opts(shape, dx, bc_lo, bc_hi, nlevels, rel_eps, abs_eps, max_vcycles, nu1, nu2, nub,
              bottom_eps, bottom_max_iter, False, threads)
    st = OrcStats()
    al = _f64f(alpha) if alpha is not None else None
    lib().orc_mac_multigrid(ctypes.byref(o), _ptr(rh), _ptr(phi), _ptr(b[0]), _ptr(b[1]),
                            _ptr(b[2] if dm == 3 else None), _ptr(al), ctypes.byref(st))
    return phi, st.as_dict()


def apply_op(u, beta, dx, bc_lo, bc_hi, alpha=None):
    """(alpha - div beta grad) u on one level (no MG)."""
    u = _f64f(u)
    shape = u.shape
    dm = len(shape)
    b = [_f64f(x) for x in beta]
    o = _opts(shape, dx, bc_lo, bc_hi, 1, 0, 0, 0, 0, 0, 0, 0, 0, False, 0)
    out = np.zeros(shape, order="F")
    al = _f64f(alpha) if alpha is not None else None
    lib().orc_apply_op(ctypes.byref(o), _ptr(u), _ptr(b[0]), _ptr(b[1]),
                       _ptr(b[2] if dm == 3 else None), _ptr(al), _ptr(out))
    return out


def mac_coeffs(rho, dx, bc_lo, bc_hi, beta0=None, beta0_edge=None, alt_energy_fix=False):
    """Face coefficients beta0^p * 2/(rho_L + rho_R) (mk_mac_coeffs + the beta0 multiply)."""
    rho = _f64f(rho)
    shape = rho.shape
    dm = len(shape)
    o = _opts(shape, dx, bc_lo, bc_hi, 1, 0, 0, 0, 0, 0, 0, 0, 0, alt_energy_fix, 0)
    out = []
    for d in range(dm):
        s = list(shape)
        s[d] += 1
        out.append(np.zeros(s, order="F"))
    b0 = np.ascontiguousarray(beta0, dtype=np.float64) if beta0 is not None else None
    b0e = np.ascontiguousarray(beta0_edge, dtype=np.float64) if beta0_edge is not None else None
    lib().orc_mac_coeffs(ctypes.byref(o), _ptr(rho), _ptr(b0), _ptr(b0e), _ptr(out[0]),
                         _ptr(out[1]), _ptr(out[2] if dm == 3 else None))
    return out


def cell_to_edge(s0_cell):
    """beta0 cell -> edge values, Source/cell_to_edge.f90:14-70 (one level)."""
    c = np.ascontiguousarray(s0_cell, dtype=np.float64)
    e = np.zeros(c.size + 1)
    lib().orc_cell_to_edge(int(c.size), _ptr(c), _ptr(e))
    return e


def make_macrhs(S_cc, delta_gamma1_term, Sbar, beta0, gamma1bar=None, p0=None, delta_p_term=None,
                delta_chi=None, dt=0.0, dpdt_factor=0.0, base_cutoff_density_coord=None,
                is_predictor=True):
    """Planar make_macrhs on whole-domain arrays (numpy restatement).

    Source/make_macrhs.f90:135-178 (2-D) and :184-240 (3-D): rhs = beta0(r) (S_cc - Sbar(r) +
    delta_gamma1_term), r the vertical (last) index; with dpdt_factor > 0, delta_chi is zeroed on
    a predictor call and, for r < base_cutoff_density_coord, delta_chi += dpdt_factor delta_p_term
    / (dt gamma1bar(r) p0(r)) and rhs += beta0(r) delta_chi.  Returns (rhs, delta_chi)."""
    S = np.asarray(S_cc, dtype=np.float64)
    shp = [1] * S.ndim
    shp[-1] = -1
    col = lambda v: np.asarray(v, dtype=np.float64).reshape(shp)  # noqa: E731
    rhs = col(beta0) * (S - col(Sbar) + np.asarray(delta_gamma1_term, dtype=np.float64))
    chi = None if delta_chi is None else np.array(delta_chi, dtype=np.float64, order="F")
    if dpdt_factor > 0.0:
        nr = S.shape[-1]
        cut = nr if base_cutoff_density_coord is None else int(base_cutoff_density_coord)
        if is_predictor:
            chi[...] = 0.0
        below = (np.arange(nr) < cut).reshape(shp)
        inc = dpdt_factor * np.asarray(delta_p_term, dtype=np.float64) / (
            dt * col(gamma1bar) * col(p0))
        chi = np.where(below, chi + inc, chi)
        rhs = np.where(below, rhs + col(beta0) * chi, rhs)
    return np.asfortranarray(rhs), (None if chi is None else np.asfortranarray(chi))


def make_at_halftime(sold, snew):
    """Source/make_at_halftime.f90:134-190: half = (old + new) / 2 cell by cell."""
    return 0.5 * (np.asarray(sold, dtype=np.float64) + np.asarray(snew, dtype=np.float64))


# ---------------------------------------------------------------- multi-level (AMR) composite

def _ml_layout(shape0, boxes):
    """nboxes / boxes int arrays of the C entry points.  `boxes[l]` (l >= 1) is a list of
    (lo, hi) tuples in level-l cell indices; boxes[0] is ignored (level 0 is the domain)."""
    nlev = len(boxes)
    dm = len(shape0)
    nb = np.zeros(nlev, dtype=np.int32)
    flat = []
    for l in range(1, nlev):
        nb[l] = len(boxes[l])
        for lo, hi in boxes[l]:
            flat += list(lo) + [0] * (3 - dm) + list(hi) + [0] * (3 - dm)
    bx = np.asarray(flat if flat else [0], dtype=np.int32)
    return nb, bx


def _ptr_array(arrs):
    t = ctypes.POINTER(ctypes.c_double) * len(arrs)
    return t(*[_ptr(a) for a in arrs])


def level_shape(shape0, l):
    return tuple(int(n) << l for n in shape0)


def ml_rel_eps(nlev: int) -> float:
    """rel_solver_eps of Source/macproject.f90:217 for nlev AMR levels."""
    return min(EPS_MAC * MAC_LEVEL_FACTOR ** (nlev - 1), EPS_MAC_MAX)


def ml_solve(rh, phi, beta, dx, bc_lo, bc_hi, boxes, nlevels=None, rel_eps=None, abs_eps=-1.0,
             max_vcycles=200, nu1=2, nu2=2, nub=10, bottom_eps=EPS_MAC_BOTTOM,
             bottom_max_iter=200, threads=0):
    """Composite multi-level solve of -div(beta grad phi) = rh (mac_oracle_ml.cpp).

    rh[l], phi[l]: cell arrays over the whole level-l domain (shape0 << l); beta[l]: list of
    face arrays of level l.  Returns (phi list, stats); covered cells of phi hold the mean of
    their children."""
    nlev = len(rh)
    shape0 = np.shape(rh[0])
    dm = len(shape0)
    rh = [_f64f(r) for r in rh]
    phi = [_f64f(p).copy(order="F") for p in phi]
    bl = []
    for l in range(nlev):
        for d in range(3):
            bl.append(_f64f(beta[l][d]) if d < dm else None)
    if nlevels is None:
        nlevels = nlevels_for_boxes([shape0])
    if rel_eps is None:
        rel_eps = ml_rel_eps(nlev)
    o = _opts(shape0, dx, bc_lo, bc_hi, nlevels, rel_eps, abs_eps, max_vcycles, nu1, nu2, nub,
              bottom_eps, bottom_max_iter, False, threads)
    nb, bx = _ml_layout(shape0, boxes)
    st = OrcStats()
    rc = lib().orc_ml_solve(ctypes.byref(o), nlev, nb.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                            bx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _ptr_array(rh),
                            _ptr_array(phi), _ptr_array(bl), ctypes.byref(st))
    if rc < 0:
        raise ValueError("invalid AMR layout (alignment or proper nesting)")
    return phi, st.as_dict()


def ml_residual(rh, phi, beta, dx, bc_lo, bc_hi, boxes):
    """Composite residual rh - L phi on every level.  Returns (list of arrays, max over valid
    cells)."""
    nlev = len(rh)
    shape0 = np.shape(rh[0])
    dm = len(shape0)
    rh = [_f64f(r) for r in rh]
    phi = [_f64f(p) for p in phi]
    res = [np.zeros(level_shape(shape0, l), order="F") for l in range(nlev)]
    bl = []
    for l in range(nlev):
        for d in range(3):
            bl.append(_f64f(beta[l][d]) if d < dm else None)
    o = _opts(shape0, dx, bc_lo, bc_hi, 1, 0, 0, 0, 0, 0, 0, 0, 0, False, 0)
    nb, bx = _ml_layout(shape0, boxes)
    r = lib().orc_ml_residual(ctypes.byref(o), nlev,
                              nb.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                              bx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _ptr_array(rh),
                              _ptr_array(phi), _ptr_array(bl), _ptr_array(res))
    if r < 0:
        raise ValueError("invalid AMR layout (alignment or proper nesting)")
    return res, float(r)


def macproject_ml(umac, phi, rho, dx, bc_lo, bc_hi, boxes, macrhs=None, beta0=None,
                  beta0_edge=None, nlevels=None, rel_eps=None, abs_eps=-1.0, max_vcycles=200,
                  nu1=2, nu2=2, nub=10, bottom_eps=EPS_MAC_BOTTOM, bottom_max_iter=200,
                  alt_energy_fix=False, threads=0):
    """Oracle multi-level MAC projection (Source/macproject.f90:51-328, nlevs > 1).

    umac[l]: list of dm face arrays over the whole level-l domain; phi[l], rho[l], macrhs[l]:
    cell arrays of level l (rho read on the level's boxes plus one ghost cell); beta0[l],
    beta0_edge[l]: planar base state of level l.  dx is the level-0 spacing.  rel_eps defaults
    to min(eps_mac 10^(nlev-1), eps_mac_max).  Returns (umac list, phi list, stats)."""
    nlev = len(phi)
    shape0 = np.shape(phi[0])
    dm = len(shape0)
    phi = [_f64f(p).copy(order="F") for p in phi]
    rho = [_f64f(r) for r in rho]
    u = [[_f64f(x).copy(order="F") for x in umac[l]] for l in range(nlev)]
    up = []
    for l in range(nlev):
        for d in range(3):
            up.append(u[l][d] if d < dm else None)
    mrl = None if macrhs is None else [None if m is None else _f64f(m) for m in macrhs]
    mr = None if mrl is None else _ptr_array(mrl)
    if beta0 is not None:
        b0 = [np.ascontiguousarray(b, dtype=np.float64) for b in beta0]
        b0e = [np.ascontiguousarray(b, dtype=np.float64) for b in beta0_edge]
        pb0, pb0e = _ptr_array(b0), _ptr_array(b0e)
    else:
        pb0 = pb0e = None
    if nlevels is None:
        nlevels = nlevels_for_boxes([shape0])
    if rel_eps is None:
        rel_eps = ml_rel_eps(nlev)
    o = _opts(shape0, dx, bc_lo, bc_hi, nlevels, rel_eps, abs_eps, max_vcycles, nu1, nu2, nub,
              bottom_eps, bottom_max_iter, alt_energy_fix, threads)
    nb, bx = _ml_layout(shape0, boxes)
    st = OrcStats()
    rc = lib().orc_macproject_ml(ctypes.byref(o), nlev,
                                 nb.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                 bx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _ptr_array(up),
                                 _ptr_array(phi), _ptr_array(rho), mr, pb0, pb0e,
                                 ctypes.byref(st))
    if rc < 0:
        raise ValueError("invalid AMR layout (alignment or proper nesting)")
    return u, phi, st.as_dict()


def create_umac_grown_fab(uf, uc, inm, d, lo, hi, ng, per):
    """create_umac_grown (Source/macproject.f90:264-272) for one face fab of a fine level.

    FBoxLib's routine is not in the MAESTRO tree; restated from its purpose: a ghost face that
    borders a cell of the fine level (inm: its cell mask over the level domain; periodic images
    wrapped) takes the fine level's value uf (the fill_boundary it ends with), any other ghost
    face the coarse level's uc after the edge restriction -- piecewise constant across the face,
    linear along its normal (mean of the two coarse faces around a fine face between coarse
    planes).  uf, uc: whole-level face arrays normal to d.  Returns the fab (box lo..hi, ng
    ghosts) with those ghost faces filled; NaN on the box's own faces and beyond a non-periodic
    domain face (the caller's physical-boundary fill)."""
    dm = len(lo)
    n = inm.shape
    shape = tuple(hi[e] - lo[e] + 1 + 2 * ng + (1 if e == d else 0) for e in range(dm))
    out = np.full(shape, np.nan)
    for a in np.ndindex(*shape):
        g = [lo[e] - ng + a[e] for e in range(dm)]
        if all(lo[e] <= g[e] <= hi[e] + (1 if e == d else 0) for e in range(dm)):
            continue
        ok = True
        for e in range(dm):
            top = n[e] if e == d else n[e] - 1
            if g[e] < 0 or g[e] > top:
                if not per[e]:
                    ok = False
                    break
                g[e] = g[e] + n[e] if g[e] < 0 else g[e] - n[e]
        if not ok:
            continue
        own = False
        for s in (0, 1):
            cc = list(g)
            cc[d] = g[d] - 1 + s
            if cc[d] < 0 or cc[d] >= n[d]:
                if not per[d]:
                    continue
                cc[d] %= n[d]
            own = own or bool(inm[tuple(cc)])
        if own:
            out[a] = uf[tuple(g)]
            continue
        c = [v // 2 for v in g]
        if g[d] % 2 == 0:
            c[d] = g[d] // 2
            out[a] = uc[tuple(c)]
        else:
            c0, c1 = list(c), list(c)
            c0[d], c1[d] = (g[d] - 1) // 2, (g[d] + 1) // 2
            out[a] = 0.5 * (uc[tuple(c0)] + uc[tuple(c1)])
    return out


# ------------------------------------------------------------------------- nodal (HG) projection

# proj_type values (Source/proj_parameters.f90)
HG_INITIAL, HG_DIVU_ITERS, HG_PRESSURE_ITERS, HG_REGULAR = 1, 2, 3, 4
# Source/mg_eps.f90:26-30
EPS_HG, EPS_HG_MAX, HG_LEVEL_FACTOR, EPS_HG_BOTTOM = 1e-12, 1e-10, 10.0, 1e-4


def _hg_opts(shape, dx, bc_lo, bc_hi, dense=True, proj_type=HG_INITIAL, dt=1.0,
             alt_energy_fix=False, rel_eps=EPS_HG, max_vcycles=100, nu1=2, nu2=2,
             bottom_eps=EPS_HG_BOTTOM, threads=0):
    dm = len(shape)
    o = OrcHgOpts()
    o.dm = dm
    for d in range(3):
        o.n[d] = int(shape[d]) if d < dm else 1
        o.dx[d] = float(dx[d]) if d < dm else 1.0
        o.bc_lo[d] = int(bc_lo[d]) if d < dm else BC_NEU
        o.bc_hi[d] = int(bc_hi[d]) if d < dm else BC_NEU
    o.dense = int(bool(dense))
    o.proj_type = int(proj_type)
    o.dt = float(dt)
    o.alt_energy_fix = int(bool(alt_energy_fix))
    o.rel_eps = float(rel_eps)
    o.max_vcycles = int(max_vcycles)
    o.nu1, o.nu2 = int(nu1), int(nu2)
    o.bottom_eps = float(bottom_eps)
    o.nthreads = int(threads)
    for f in range(6):
        o.wall_off[f] = -1
    o.wall = None
    return o


def hg_wall_layout(shape, inflow_lo, inflow_hi):
    """Offsets of the inflow faces in a wall array: face f = 2 d + side in that order, each
    holding its cells (the face's other directions, Fortran order).  Returns (offsets, total)."""
    dm = len(shape)
    off, tot = [-1] * 6, 0
    for f in range(2 * dm):
        d, side = divmod(f, 2)
        if not (inflow_hi if side else inflow_lo)[d]:
            continue
        off[f] = tot
        tot += int(np.prod([shape[e] for e in range(dm) if e != d]))
    return off, tot


def hg_wall_from_ghosts(shape, inflow_lo, inflow_hi, proj_type, dt, unew_pad, uold_pad=None,
                        beta0_pad=None):
    """The inflow faces' wall values of beta0 U_d as hgproject leaves the ghost cells outside
    them: `*_pad` are whole-domain arrays with one ghost layer (cells + 2 per direction; unew /
    uold with a trailing component axis).  create_uvec_for_projection forms (U - Uold) / dt on
    the first ghost layer too for the pressure iterations and leaves an inlet's ghost cells
    otherwise as filled (Source/hgproject.f90:461-474, 500-511: only walls and symmetry faces are
    zeroed); U is then multiplied by beta0_cart on beta0_cart's ghost layers
    (Source/hgproject.f90:140-143; beta0_pad None: beta0_cart has no ghost layer, no scaling)."""
    dm = len(shape)
    off, tot = hg_wall_layout(shape, inflow_lo, inflow_hi)
    wall = np.zeros(max(tot, 1))
    for f in range(2 * dm):
        if off[f] < 0:
            continue
        d, side = divmod(f, 2)
        sl = [slice(1, shape[e] + 1) for e in range(dm)]
        sl[d] = 0 if side == 0 else shape[d] + 1
        sl = tuple(sl)
        w = np.asarray(unew_pad)[sl + (d,)].astype(np.float64)
        if proj_type == HG_PRESSURE_ITERS:
            w = (w - np.asarray(uold_pad)[sl + (d,)]) / dt
        if beta0_pad is not None:
            w = w * np.asarray(beta0_pad)[sl]
        m = w.size
        wall[off[f]:off[f] + m] = np.ravel(w, order="F")
    return wall


def node_shape(shape):
    return tuple(int(v) + 1 for v in shape)


def hg_apply(sigma, phi, dx, bc_lo, bc_hi, dense=True):
    """Nodal operator L phi (cell coefficients sigma, node array phi)."""
    sigma = _f64f(sigma)
    phi = _f64f(phi)
    o = _hg_opts(sigma.shape, dx, bc_lo, bc_hi, dense=dense)
    out = np.zeros(node_shape(sigma.shape), order="F")
    lib().orc_hg_apply(ctypes.byref(o), _ptr(sigma), _ptr(phi), _ptr(out))
    return out


def hg_divu(u, dx, bc_lo, bc_hi):
    """Node-centred divergence of a cell vector field u (shape cells + (dm,))."""
    u = _f64f(u)
    shape = u.shape[:-1]
    o = _hg_opts(shape, dx, bc_lo, bc_hi)
    out = np.zeros(node_shape(shape), order="F")
    lib().orc_hg_divu(ctypes.byref(o), _ptr(u), _ptr(out))
    return out


def hg_grad(phi, dx, bc_lo, bc_hi):
    """Cell gradient of a nodal field (mkgphi); returns shape cells + (dm,)."""
    phi = _f64f(phi)
    shape = tuple(v - 1 for v in phi.shape)
    o = _hg_opts(shape, dx, bc_lo, bc_hi)
    g = np.zeros(shape + (len(shape),), order="F")
    lib().orc_hg_grad(ctypes.byref(o), _ptr(phi), _ptr(g))
    return g


def hg_solve(sigma, rh, dx, bc_lo, bc_hi, phi=None, dense=True, rel_eps=EPS_HG,
             max_vcycles=100, threads=0):
    """Nodal solve L phi = rh.  Returns (phi, stats)."""
    sigma = _f64f(sigma)
    rh = _f64f(rh)
    phi = np.zeros(rh.shape, order="F") if phi is None else _f64f(phi).copy(order="F")
    o = _hg_opts(sigma.shape, dx, bc_lo, bc_hi, dense=dense, rel_eps=rel_eps,
                 max_vcycles=max_vcycles, threads=threads)
    st = OrcStats()
    lib().orc_hg_solve(ctypes.byref(o), _ptr(sigma), _ptr(rh), _ptr(phi), ctypes.byref(st))
    return phi, st.as_dict()


def hgproject(unew, uold, gpi, rhohalf, pi, dx, bc_lo, bc_hi, proj_type=HG_REGULAR, dt=1.0,
              beta0_cart=None, nodalrhs=None, dense=True, alt_energy_fix=False, rel_eps=EPS_HG,
              max_vcycles=100, threads=0, inflow_lo=(0, 0, 0), inflow_hi=(0, 0, 0), wall=None):
    """Oracle nodal projection on one level (Source/hgproject.f90:32-264).

    Cell vector fields unew / uold / gpi have shape cells + (dm,); rhohalf and beta0_cart are
    cell arrays; pi and nodalrhs node arrays (cells + 1 per direction).  Inlet faces:
    inflow_lo / inflow_hi flags with `wall` their wall values (hg_wall_from_ghosts).  Returns
    (unew, gpi, pi, phi, stats)."""
    unew = _f64f(unew).copy(order="F")
    gpi = _f64f(gpi).copy(order="F")
    pi = _f64f(pi).copy(order="F")
    uold = _f64f(uold)
    rhohalf = _f64f(rhohalf)
    shape = rhohalf.shape
    b0 = None if beta0_cart is None else _f64f(beta0_cart)
    nr = None if nodalrhs is None else _f64f(nodalrhs)
    phi = np.zeros(node_shape(shape), order="F")
    o = _hg_opts(shape, dx, bc_lo, bc_hi, dense=dense, proj_type=proj_type, dt=dt,
                 alt_energy_fix=alt_energy_fix, rel_eps=rel_eps, max_vcycles=max_vcycles,
                 threads=threads)
    off, tot = hg_wall_layout(shape, inflow_lo, inflow_hi)
    if tot > 0:
        wall = _f64f(wall)
        if wall.size < tot:
            raise ValueError("wall array shorter than the inflow faces")
        for f in range(6):
            o.wall_off[f] = off[f]
        o.wall = wall.ctypes.data
    st = OrcStats()
    lib().orc_hgproject(ctypes.byref(o), _ptr(unew), _ptr(uold), _ptr(gpi), _ptr(rhohalf),
                        _ptr(pi), _ptr(b0), _ptr(nr), _ptr(phi), ctypes.byref(st))
    return unew, gpi, pi, phi, st.as_dict()
