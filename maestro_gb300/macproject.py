"""Host-side mirror of MAESTRO's MAC-projection interface over the GB300 C ABI.

Mirrors, with the reference's names and argument meaning:

* ``macproject(umac, phi, rho, dx, the_bc_tower, macrhs, beta0_1d, beta0_1d_edge)``
  -- Source/macproject.f90:51-76 (single level; the multifab arguments are lists of per-box
  Fortran-ordered numpy fabs, see ``Layout``);
* ``mac_multigrid(rh, phi, solver_alpha, solver_beta, dx, the_bc_tower, rel_solver_eps,
  abs_solver_eps)`` -- Source/mac_multigrid.f90:18-37;
* ``cell_to_edge(s0_cell)`` -- Source/cell_to_edge.f90:14.

Errors: the reference aborts through ``bl_error``; here every C status other than MAC_OK raises
``MacError`` (carrying the code), except MAC_ERR_NOT_CONVERGED, which is reported in the
returned statistics unless ``strict=True``.
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np

from . import capi
from .capi import MacError

BC_PER, BC_INT, BC_DIR, BC_NEU = capi.MAC_BC_PER, capi.MAC_BC_INT, capi.MAC_BC_DIR, capi.MAC_BC_NEU


@dataclasses.dataclass
class BcTower:
    """The press_comp slice of MAESTRO's bc_tower: elliptic BC per direction and side
    (ell_bc_level_array(..., press_comp), Source/define_bc_tower.f90:296-400)."""

    lo: tuple
    hi: tuple

    @staticmethod
    def from_phys(phys_lo, phys_hi):
        """Map physical BC names to the press_comp elliptic BCs (Source/define_bc_tower.f90:
        slip/no-slip wall, inlet, symmetry -> Neumann; outlet -> Dirichlet; periodic)."""
        m = {"periodic": BC_PER, "slip wall": BC_NEU, "no slip wall": BC_NEU, "inlet": BC_NEU,
             "symmetry": BC_NEU, "outlet": BC_DIR}
        return BcTower(tuple(m[p] for p in phys_lo), tuple(m[p] for p in phys_hi))


class Layout:
    """Single-level box layout: the boxes of an ml_layout level (0-based inclusive lo/hi)."""

    def __init__(self, domain_n, boxes):
        self.n = tuple(int(v) for v in domain_n)
        self.dm = len(self.n)
        self.boxes = [(tuple(lo), tuple(hi)) for lo, hi in boxes]

    @staticmethod
    def tiled(domain_n, box):
        n = tuple(domain_n)
        dm = len(n)
        nb = [n[d] // box[d] for d in range(dm)]
        out = []
        for idx in np.ndindex(*reversed(nb)):
            idx = tuple(reversed(idx))
            lo = tuple(idx[d] * box[d] for d in range(dm))
            hi = tuple(lo[d] + box[d] - 1 for d in range(dm))
            out.append((lo, hi))
        return Layout(n, out)

    # ---- global <-> per-box fabs (Fortran order, ghosts filled periodically / by clamping) ----
    def to_fabs(self, arr, ng=0, face_dir=None, periodic=None, ncomp=1):
        """Split a whole-domain array into per-box fabs with `ng` ghosts.

        face_dir: None for cell data, d for faces normal to d (one extra entry along d).
        Ghosts: periodic wrap where `periodic[d]`, else clamped to the nearest valid entry.
        ncomp > 1: the array has a trailing component axis.
        """
        periodic = periodic or [False] * self.dm
        arr = np.asarray(arr)
        fabs = []
        for lo, hi in self.boxes:
            idx = []
            for d in range(self.dm):
                extra = 1 if face_dir == d else 0
                r = np.arange(lo[d] - ng, hi[d] + 1 + extra + ng)
                lim = self.n[d] + extra
                if periodic[d]:
                    r = np.where(r < 0, r + self.n[d], r)
                    r = np.where(r >= lim, r - self.n[d], r)
                else:
                    r = np.clip(r, 0, lim - 1)
                idx.append(r)
            sub = arr[np.ix_(*idx)] if ncomp == 1 else arr[np.ix_(*idx, np.arange(ncomp))]
            fabs.append(np.asfortranarray(sub, dtype=np.float64))
        return fabs

    def from_fabs(self, fabs, ng=0, face_dir=None):
        """Whole-domain array from the valid region of per-box fabs."""
        shape = list(self.n)
        if face_dir is not None:
            shape[face_dir] += 1
        out = np.zeros(shape, order="F")
        for (lo, hi), f in zip(self.boxes, fabs):
            dst, src = [], []
            for d in range(self.dm):
                extra = 1 if face_dir == d else 0
                dst.append(slice(lo[d], hi[d] + 1 + extra))
                src.append(slice(ng, ng + hi[d] - lo[d] + 1 + extra))
            out[tuple(dst)] = f[tuple(src)]
        return out


def _ptr_array(arrs):
    """ctypes double** over a list of float64 Fortran-contiguous numpy arrays."""
    P = ctypes.POINTER(ctypes.c_double)
    a = (P * len(arrs))()
    for i, x in enumerate(arrs):
        assert x.dtype == np.float64 and x.flags.f_contiguous, "fabs must be float64, Fortran order"
        a[i] = x.ctypes.data_as(P)
    return a


def _dptr(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(
        ctypes.POINTER(ctypes.c_double))


class MacProjector:
    """A solver context bound to one level geometry (mac_ctx_create / mac_ctx_destroy)."""

    def __init__(self, layout: Layout, dx, bc: BcTower, precision="fp64", stream=None, **opts):
        self.layout = layout
        self.dm = layout.dm
        g = capi.MacGeom()
        g.dm = self.dm
        for d in range(3):
            g.domain_lo[d] = 0
            g.domain_hi[d] = layout.n[d] - 1 if d < self.dm else 0
            g.dx[d] = float(dx[d]) if d < self.dm else 1.0
            g.bc_lo[d] = int(bc.lo[d]) if d < self.dm else BC_NEU
            g.bc_hi[d] = int(bc.hi[d]) if d < self.dm else BC_NEU
        nb = len(layout.boxes)
        self._blo = (ctypes.c_int * (3 * nb))()
        self._bhi = (ctypes.c_int * (3 * nb))()
        for b, (lo, hi) in enumerate(layout.boxes):
            for d in range(3):
                self._blo[3 * b + d] = lo[d] if d < self.dm else 0
                self._bhi[3 * b + d] = hi[d] if d < self.dm else 0
        g.nboxes = nb
        g.box_lo = ctypes.cast(self._blo, ctypes.POINTER(ctypes.c_int))
        g.box_hi = ctypes.cast(self._bhi, ctypes.POINTER(ctypes.c_int))
        self.geom = g
        self.bc = bc
        self.opts = capi.default_opts(
            precision=capi.MAC_PREC_MIXED if precision == "mixed" else capi.MAC_PREC_FP64, **opts)
        self.ctx = ctypes.c_void_p()
        rc = capi.lib().mac_ctx_create(ctypes.byref(self.ctx), ctypes.byref(g),
                                       ctypes.byref(self.opts), ctypes.c_void_p(stream or 0))
        if rc != capi.MAC_OK:
            raise MacError(rc, "mac_ctx_create")

    def close(self):
        if self.ctx:
            capi.lib().mac_ctx_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_opts(self, **kw):
        for k, v in kw.items():
            if k == "precision" and isinstance(v, str):
                v = capi.MAC_PREC_MIXED if v == "mixed" else capi.MAC_PREC_FP64
            setattr(self.opts, k, v)
        rc = capi.lib().mac_ctx_set_opts(self.ctx, ctypes.byref(self.opts))
        if rc != capi.MAC_OK:
            raise MacError(rc, "mac_ctx_set_opts")

    def levels(self):
        buf = (ctypes.c_int * (3 * 32))()
        n = capi.lib().mac_ctx_levels(self.ctx, buf)
        return [tuple(buf[3 * l + d] for d in range(3)) for l in range(n)]

    @staticmethod
    def _check(rc, where, st, strict):
        if rc == capi.MAC_OK or (rc == capi.MAC_ERR_NOT_CONVERGED and not strict):
            return
        raise MacError(rc, where)

    def macproject(self, umac, phi, rho, macrhs=None, beta0_1d=None, beta0_1d_edge=None,
                   ng_u=1, ng_phi=1, ng_rho=1, ng_rhs=0, rho_ncomp=1, rho_comp=0, strict=False):
        """MAC-project per-box fabs in place (Source/macproject.f90:51-328).

        umac: list over directions of lists over boxes of edge fabs; phi, rho, macrhs: lists
        over boxes.  Returns the solver statistics (dict)."""
        nb = len(self.layout.boxes)
        flat_u = [umac[d][b] for d in range(self.dm) for b in range(nb)]
        st = capi.MacStats()
        rc = capi.lib().mac_macproject(
            self.ctx, capi.MAC_PTR_HOST, _ptr_array(flat_u), ng_u, _ptr_array(phi), ng_phi,
            _ptr_array(rho), ng_rho, rho_ncomp, rho_comp,
            _ptr_array(macrhs) if macrhs is not None else None, ng_rhs,
            _dptr(beta0_1d), _dptr(beta0_1d_edge), ctypes.byref(st))
        self._check(rc, "mac_macproject", st, strict)
        return st.as_dict()

    def macproject_cart(self, umac, phi, rho, beta0_cart_edge, macrhs=None, ng_u=1, ng_phi=1,
                        ng_rho=1, ng_rhs=0, ng_b=1, rho_ncomp=1, rho_comp=0, strict=False):
        """Spherical form of macproject on per-box fabs in place: beta0 on every face
        (beta0_cart_edge: list over directions of lists over boxes of edge fabs)."""
        nb = len(self.layout.boxes)
        flat_u = [umac[d][b] for d in range(self.dm) for b in range(nb)]
        flat_b = [beta0_cart_edge[d][b] for d in range(self.dm) for b in range(nb)]
        st = capi.MacStats()
        rc = capi.lib().mac_macproject_cart(
            self.ctx, capi.MAC_PTR_HOST, _ptr_array(flat_u), ng_u, _ptr_array(phi), ng_phi,
            _ptr_array(rho), ng_rho, rho_ncomp, rho_comp,
            _ptr_array(macrhs) if macrhs is not None else None, ng_rhs, _ptr_array(flat_b),
            ng_b, ctypes.byref(st))
        self._check(rc, "mac_macproject_cart", st, strict)
        return st.as_dict()

    def mac_multigrid(self, rh, phi, solver_beta, solver_alpha=None, ng_rh=0, ng_phi=1,
                      ng_alpha=1, ng_beta=1, strict=False):
        """Solve (alpha - div beta grad) phi = rh on per-box fabs (Source/mac_multigrid.f90)."""
        nb = len(self.layout.boxes)
        flat_b = [solver_beta[d][b] for d in range(self.dm) for b in range(nb)]
        st = capi.MacStats()
        rc = capi.lib().mac_multigrid(
            self.ctx, capi.MAC_PTR_HOST, _ptr_array(rh), ng_rh, _ptr_array(phi), ng_phi,
            _ptr_array(solver_alpha) if solver_alpha is not None else None, ng_alpha,
            _ptr_array(flat_b), ng_beta, ctypes.byref(st))
        self._check(rc, "mac_multigrid", st, strict)
        return st.as_dict()

    def make_macrhs(self, macrhs, S_cc, delta_gamma1_term, Sbar, beta0, gamma1bar=None, p0=None,
                    delta_p_term=None, delta_chi=None, dt=0.0, dpdt_factor=0.0,
                    base_cutoff_density_coord=None, is_predictor=True, ng_rh=0, ng_sr=0, ng_dg=0,
                    ng_dp=0, ng_d=0):
        """Per-box make_macrhs (Source/make_macrhs.f90:28-240, planar); fills macrhs (and updates
        delta_chi) in place.  base_cutoff_density_coord defaults to the vertical extent."""
        nr = self.layout.n[-1]
        cut = nr if base_cutoff_density_coord is None else int(base_cutoff_density_coord)
        chi = dpdt_factor > 0.0
        rc = capi.lib().mac_make_macrhs(
            self.ctx, capi.MAC_PTR_HOST, _ptr_array(macrhs), ng_rh, _ptr_array(S_cc), ng_sr,
            _ptr_array(delta_gamma1_term), ng_dg, _dptr(Sbar), _dptr(beta0),
            _dptr(gamma1bar) if chi else None, _dptr(p0) if chi else None,
            _ptr_array(delta_p_term) if chi else None, ng_dp,
            _ptr_array(delta_chi) if chi else None, ng_d, float(dt), float(dpdt_factor), cut,
            int(bool(is_predictor)))
        if rc != capi.MAC_OK:
            raise MacError(rc, "mac_make_macrhs")

    def make_at_halftime(self, half, sold, snew, in_comp=0, s_ncomp=1, ng_half=1, ng_old=1,
                         ng_new=1):
        """Per-box make_at_halftime (Source/make_at_halftime.f90:82-130); fills half in place."""
        rc = capi.lib().mac_make_at_halftime(
            self.ctx, capi.MAC_PTR_HOST, _ptr_array(half), ng_half, 0, 1, _ptr_array(sold), ng_old,
            _ptr_array(snew), ng_new, int(in_comp), int(s_ncomp))
        if rc != capi.MAC_OK:
            raise MacError(rc, "mac_make_at_halftime")

    def macproject_dense(self, ux, uy, uz, phi, rho, macrhs=None, beta0=None, beta0_edge=None,
                         strict=False):
        """Whole-domain variant on device pointers (ints, e.g. torch tensor data_ptr())."""
        st = capi.MacStats()
        v = ctypes.c_void_p
        rc = capi.lib().mac_macproject_dense(
            self.ctx, v(ux), v(uy), v(uz or 0), v(phi), v(rho), v(macrhs or 0), v(beta0 or 0),
            v(beta0_edge or 0), ctypes.byref(st))
        self._check(rc, "mac_macproject_dense", st, strict)
        return st.as_dict()

    def macproject_cart_dense(self, ux, uy, uz, phi, rho, b0x, b0y, b0z, macrhs=None,
                              strict=False):
        """Whole-domain spherical form on device pointers (ints)."""
        st = capi.MacStats()
        v = ctypes.c_void_p
        rc = capi.lib().mac_macproject_cart_dense(
            self.ctx, v(ux), v(uy), v(uz or 0), v(phi), v(rho), v(macrhs or 0), v(b0x), v(b0y),
            v(b0z or 0), ctypes.byref(st))
        self._check(rc, "mac_macproject_cart_dense", st, strict)
        return st.as_dict()

    def set_amr(self, boxes):
        """Multi-level hierarchy (mac_ctx_set_amr): boxes[l] for l >= 1 is a list of (lo, hi)
        inclusive corners in level-l cell indices (ratio 2); boxes[0] is ignored (level 0 is
        this projector's layout).  A list of one level drops the hierarchy."""
        nlev = len(boxes)
        dm = self.dm
        nb = (ctypes.c_int * max(1, nlev))()
        lo, hi = [], []
        for l in range(1, nlev):
            nb[l] = len(boxes[l])
            for a, b in boxes[l]:
                lo += list(a) + [0] * (3 - dm)
                hi += list(b) + [0] * (3 - dm)
        clo = (ctypes.c_int * max(1, len(lo)))(*lo)
        chi = (ctypes.c_int * max(1, len(hi)))(*hi)
        rc = capi.lib().mac_ctx_set_amr(self.ctx, nlev, nb, clo, chi)
        if rc != 0:
            raise MacError(rc, "mac_ctx_set_amr")
        self.amr_levels = nlev

    def macproject_ml_dense(self, umac, phi, rho, macrhs=None, beta0=None, beta0_edge=None,
                            strict=False):
        """Multi-level projection on whole-level-domain device arrays (ints: device pointers):
        umac[l] a list of dm face arrays, phi[l], rho[l], macrhs[l] (or None) cells, beta0[l] /
        beta0_edge[l] the planar base state of level l."""
        nlev = len(phi)
        dm = self.dm
        v = ctypes.c_void_p
        U = (v * (3 * nlev))(*[(umac[l][d] if d < dm else 0) for l in range(nlev) for d in range(3)])
        Ph = (v * nlev)(*phi)
        R = (v * nlev)(*rho)
        M = None if macrhs is None else (v * nlev)(*[(m or 0) for m in macrhs])
        B0 = None if beta0 is None else (v * nlev)(*beta0)
        B0e = None if beta0_edge is None else (v * nlev)(*beta0_edge)
        st = capi.MacStats()
        rc = capi.lib().mac_macproject_ml_dense(self.ctx, U, Ph, R, M, B0, B0e, ctypes.byref(st))
        self._check(rc, "mac_macproject_ml_dense", st, strict)
        return st.as_dict()

    def macproject_ml(self, umac, phi, rho, macrhs=None, beta0=None, beta0_edge=None, ng_u=1,
                      ng_phi=1, ng_rho=1, ng_rhs=0, rho_ncomp=1, rho_comp=0, strict=False):
        """Multi-level MAC projection of per-box host fabs in place (mac_macproject_ml; needs
        set_amr).  umac[l][d][b], phi[l][b], rho[l][b], macrhs[l][b] (or None) for every level
        l; beta0[l] / beta0_edge[l] the planar base state of level l (or None)."""
        nlev = len(phi)
        flat_u, flat_p, flat_r, flat_m = [], [], [], []
        for l in range(nlev):
            nb = len(phi[l])
            flat_u += [umac[l][d][b] for d in range(self.dm) for b in range(nb)]
            flat_p += list(phi[l])
            flat_r += list(rho[l])
            if macrhs is not None:
                flat_m += list(macrhs[l])
        b0 = None if beta0 is None else np.concatenate([np.asarray(b, dtype=np.float64)
                                                        for b in beta0])
        b0e = None if beta0_edge is None else np.concatenate([np.asarray(b, dtype=np.float64)
                                                              for b in beta0_edge])
        st = capi.MacStats()
        rc = capi.lib().mac_macproject_ml(
            self.ctx, capi.MAC_PTR_HOST, _ptr_array(flat_u), ng_u, _ptr_array(flat_p), ng_phi,
            _ptr_array(flat_r), ng_rho, rho_ncomp, rho_comp,
            _ptr_array(flat_m) if macrhs is not None else None, ng_rhs, _dptr(b0), _dptr(b0e),
            ctypes.byref(st))
        self._check(rc, "mac_macproject_ml", st, strict)
        return st.as_dict()

    def set_inflow(self, lo_inflow=(0, 0, 0), hi_inflow=(0, 0, 0)):
        """Inlet faces of the nodal projection (mac_ctx_set_inflow): flags per direction."""
        lo = (ctypes.c_int * 3)(*(list(lo_inflow) + [0] * (3 - len(lo_inflow))))
        hi = (ctypes.c_int * 3)(*(list(hi_inflow) + [0] * (3 - len(hi_inflow))))
        rc = capi.lib().mac_ctx_set_inflow(self.ctx, lo, hi)
        if rc != capi.MAC_OK:
            raise MacError(rc, "mac_ctx_set_inflow")

    def hgproject_dense(self, proj_type, dt, unew, uold, gpi, rhohalf, pi, beta0_cart=None,
                        nodalrhs=None, dense_stencil=True, rel_eps=1e-12, strict=False,
                        inflow_wall=None):
        """Nodal (HG) projection on this projector's domain (mac_hgproject_dense, or
        mac_hgproject_dense_inflow with the inlet faces' wall values), device pointers (ints):
        cell vector fields unew / uold / gpi (cells x dm, component-major), rhohalf and
        beta0_cart cells, pi and nodalrhs nodes (cells + 1 per direction)."""
        st = capi.MacStats()
        v = ctypes.c_void_p
        args = (self.ctx, int(proj_type), float(dt), int(bool(dense_stencil)), float(rel_eps),
                v(unew), v(uold or 0), v(gpi), v(rhohalf), v(pi), v(beta0_cart or 0),
                v(nodalrhs or 0))
        if inflow_wall is None:
            name = "mac_hgproject_dense"
            rc = capi.lib().mac_hgproject_dense(*args, ctypes.byref(st))
        else:
            name = "mac_hgproject_dense_inflow"
            rc = capi.lib().mac_hgproject_dense_inflow(*args, v(inflow_wall), ctypes.byref(st))
        self._check(rc, name, st, strict)
        return st.as_dict()

    def hgproject(self, proj_type, dt, unew, uold, gpi, rhohalf, pi, beta0_cart=None,
                  nodalrhs=None, ng_u=1, ng_uo=1, ng_gp=1, ng_rho=1, ng_pi=1, ng_b0=1, ng_nr=1,
                  dense_stencil=True, rel_eps=1e-12, strict=False):
        """Nodal (HG) projection of per-box host fabs in place (mac_hgproject): unew, uold, gpi
        cell fabs with dm components (lists over boxes), rhohalf / beta0_cart cell fabs, pi /
        nodalrhs node fabs."""
        opt = lambda a: None if a is None else _ptr_array(a)  # noqa: E731
        st = capi.MacStats()
        rc = capi.lib().mac_hgproject(
            self.ctx, capi.MAC_PTR_HOST, int(proj_type), float(dt), int(bool(dense_stencil)),
            float(rel_eps), _ptr_array(unew), ng_u, opt(uold), ng_uo, _ptr_array(gpi), ng_gp,
            _ptr_array(rhohalf), ng_rho, _ptr_array(pi), ng_pi, opt(beta0_cart), ng_b0,
            opt(nodalrhs), ng_nr, ctypes.byref(st))
        self._check(rc, "mac_hgproject", st, strict)
        return st.as_dict()

    def adjoint_dense(self, u, rho, macrhs, beta0, beta0_edge, w, du, drinv=None, dbeta0=None,
                      dmacrhs=None, phi_out=None, strict=True):
        """Adjoint of the whole-domain projection on device pointers (see maestro_mac.h)."""
        st = capi.MacStats()
        v = ctypes.c_void_p
        u3 = list(u) + [0] * (3 - len(u))
        w3 = list(w) + [0] * (3 - len(w))
        d3 = list(du) + [0] * (3 - len(du))
        rc = capi.lib().mac_macproject_adjoint_dense(
            self.ctx, v(u3[0]), v(u3[1]), v(u3[2]), v(rho), v(macrhs or 0), v(beta0 or 0),
            v(beta0_edge or 0), v(w3[0]), v(w3[1]), v(w3[2]), v(d3[0]), v(d3[1]), v(d3[2]),
            v(drinv or 0), v(dbeta0 or 0), v(dmacrhs or 0), v(phi_out or 0), ctypes.byref(st))
        self._check(rc, "mac_macproject_adjoint_dense", st, strict)
        return st.as_dict()


def macproject(umac, phi, rho, dx, the_bc_tower: BcTower, macrhs=None, beta0_1d=None,
               beta0_1d_edge=None, box=None, precision="fp64", **opts):
    """One-shot MAC projection on whole-domain numpy arrays (natural Fortran-order layout).

    Splits the arrays into boxes of extent `box` (default: one box), projects through the C ABI
    with host pointers and returns (umac_new list, phi_new, stats)."""
    phi = np.asfortranarray(phi, dtype=np.float64)
    n = phi.shape
    dm = len(n)
    lay = Layout.tiled(n, box or n)
    per = [the_bc_tower.lo[d] == BC_PER for d in range(dm)]
    fu = [lay.to_fabs(umac[d], ng=1, face_dir=d, periodic=per) for d in range(dm)]
    fphi = lay.to_fabs(phi, ng=1, periodic=per)
    frho = lay.to_fabs(rho, ng=1, periodic=per)
    frhs = lay.to_fabs(macrhs, ng=0) if macrhs is not None else None
    P = MacProjector(lay, dx, the_bc_tower, precision=precision, **opts)
    try:
        st = P.macproject(fu, fphi, frho, frhs, beta0_1d, beta0_1d_edge)
    finally:
        P.close()
    u_new = [lay.from_fabs(fu[d], ng=1, face_dir=d) for d in range(dm)]
    return u_new, lay.from_fabs(fphi, ng=1), st


def macproject_cart(umac, phi, rho, dx, the_bc_tower: BcTower, beta0_cart_edge, macrhs=None,
                    box=None, precision="fp64", **opts):
    """One-shot spherical-form MAC projection on whole-domain numpy arrays (beta0 on every
    face, one face array per direction).  Returns (umac_new list, phi_new, stats)."""
    phi = np.asfortranarray(phi, dtype=np.float64)
    n = phi.shape
    dm = len(n)
    lay = Layout.tiled(n, box or n)
    per = [the_bc_tower.lo[d] == BC_PER for d in range(dm)]
    fu = [lay.to_fabs(umac[d], ng=1, face_dir=d, periodic=per) for d in range(dm)]
    fb = [lay.to_fabs(beta0_cart_edge[d], ng=1, face_dir=d, periodic=per) for d in range(dm)]
    fphi = lay.to_fabs(phi, ng=1, periodic=per)
    frho = lay.to_fabs(rho, ng=1, periodic=per)
    frhs = lay.to_fabs(macrhs, ng=0) if macrhs is not None else None
    P = MacProjector(lay, dx, the_bc_tower, precision=precision, **opts)
    try:
        st = P.macproject_cart(fu, fphi, frho, fb, frhs)
    finally:
        P.close()
    u_new = [lay.from_fabs(fu[d], ng=1, face_dir=d) for d in range(dm)]
    return u_new, lay.from_fabs(fphi, ng=1), st


def cell_to_edge(s0_cell):
    """beta0 cell -> edge through the C ABI (Source/cell_to_edge.f90:14-70)."""
    c = np.ascontiguousarray(s0_cell, dtype=np.float64)
    e = np.zeros(c.size + 1)
    rc = capi.lib().mac_cell_to_edge(int(c.size), c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if rc != capi.MAC_OK:
        raise MacError(rc, "mac_cell_to_edge")
    return e
