"""Golden fixtures that pin the nodal (HG) projection oracle (oracle/hg_oracle.cpp).

The reference's nodal solver is the un-vendored FBoxLib (ml_nd_solve) and its repository holds no
numeric outputs for it, so the fixtures come from an MG-independent computation of the same
discrete problem, written with numpy/scipy and sharing no code with the oracle:

  * dense operator   the finite-element stiffness of each cell, computed here by 2-point Gauss
                     quadrature of the (bi/tri)linear basis gradients, times the cell coefficient
                     sigma, assembled on the nodes and divided by the nodal volume (the oracle uses
                     the closed tensor-product form); sigma = 0 outside non-periodic faces
  * cross operator   sigma on each node-to-node edge = mean of the 2^(dm-1) cells along it
  * divergence       Docs/mg/mg.tex:485-493: (DU)_node = sum_d [mean of u_d over the cells on the
                     + side - the same on the - side] / h_d, U = 0 outside non-periodic faces;
                     at an inflow face (hg_multigrid's lo_inflow / hi_inflow) the ghost cell
                     outside adds the flux of its normal velocity (the inflow on the wall)
  * solve            sparse LU on the unknown nodes (periodic images identified, outflow nodes
                     fixed at 0), the mean of phi over the unknowns pinned for the singular problem
  * hgproject        Source/hgproject.f90:32-264 (create_uvec, beta0 scaling, alt energy fix,
                     mkgphi, hg_update for the four projection types)

Run from the repository root:  python tests/golden/make_golden_hg.py
"""
from __future__ import annotations

import itertools
import os
import sys

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from maestro_gb300.inputs import BC_DIR, BC_NEU, BC_PER  # noqa: E402

HG_INITIAL, HG_DIVU_ITERS, HG_PRESSURE_ITERS, HG_REGULAR = 1, 2, 3, 4


class Nodes:
    def __init__(self, shape, dx, bc_lo, bc_hi):
        self.shape = tuple(shape)
        self.dm = len(shape)
        self.dx = tuple(dx)
        self.per = [bc_lo[d] == BC_PER for d in range(self.dm)]
        self.dlo = [bc_lo[d] == BC_DIR for d in range(self.dm)]
        self.dhi = [bc_hi[d] == BC_DIR for d in range(self.dm)]
        self.nshape = tuple(n + 1 for n in shape)
        # unknown numbering over storage nodes
        self.uid = -np.ones(self.nshape, dtype=np.int64)
        cnt = 0
        for p in itertools.product(*[range(m) for m in self.nshape]):
            if self.is_unknown(p):
                self.uid[p] = cnt
                cnt += 1
        self.nunk = cnt

    def is_unknown(self, p):
        for d in range(self.dm):
            n = self.shape[d]
            if self.per[d]:
                if p[d] == n:
                    return False
            else:
                if (p[d] == 0 and self.dlo[d]) or (p[d] == n and self.dhi[d]):
                    return False
        return True

    def fold(self, p):
        """Storage node -> the node that carries its value (periodic image), or None (fixed 0)."""
        q = list(p)
        for d in range(self.dm):
            n = self.shape[d]
            if self.per[d]:
                q[d] %= n
            elif q[d] < 0 or q[d] > n:
                return None
        q = tuple(q)
        return q if self.uid[q] >= 0 else None

    def cell(self, c):
        q = list(c)
        for d in range(self.dm):
            n = self.shape[d]
            if self.per[d]:
                q[d] %= n
            elif q[d] < 0 or q[d] >= n:
                return None
        return tuple(q)


def element_stiffness(dx):
    """FE stiffness of one cell, unit coefficient, by 2-point Gauss quadrature, divided by the
    cell volume (nodal-volume scaling).  Keys: local corner tuples."""
    dm = len(dx)
    g = [0.5 - 0.5 / np.sqrt(3.0), 0.5 + 0.5 / np.sqrt(3.0)]
    corners = list(itertools.product((0, 1), repeat=dm))
    K = np.zeros((len(corners), len(corners)))
    vol = float(np.prod(dx))
    for q in itertools.product(g, repeat=dm):
        w = vol / (2 ** dm)
        grads = []
        for a in corners:
            gr = []
            for d in range(dm):
                t = (1.0 if a[d] else -1.0) / dx[d]
                for e in range(dm):
                    if e != d:
                        t *= q[e] if a[e] else (1.0 - q[e])
                gr.append(t)
            grads.append(np.array(gr))
        for i in range(len(corners)):
            for j in range(len(corners)):
                K[i, j] += w * grads[i] @ grads[j]
    return corners, K / vol


def operator(N: Nodes, sigma, dense=True):
    """Sparse L over the unknowns (rows and columns by uid): L phi ~ div(sigma grad phi)."""
    rows, cols, vals = [], [], []
    dm = N.dm
    if dense:
        corners, K = element_stiffness(N.dx)
        for c in itertools.product(*[range(n) for n in N.shape]):
            s = sigma[c]
            for i, a in enumerate(corners):
                p = N.fold(tuple(c[d] + a[d] for d in range(dm)))
                if p is None:
                    continue
                for j, b in enumerate(corners):
                    m = N.fold(tuple(c[d] + b[d] for d in range(dm)))
                    if m is None:
                        continue
                    rows.append(N.uid[p])
                    cols.append(N.uid[m])
                    vals.append(-s * K[i, j])
    else:
        for p in itertools.product(*[range(m) for m in N.nshape]):
            if N.uid[p] < 0:
                continue
            for d in range(dm):
                for s in (-1, 1):
                    q = list(p)
                    q[d] += s
                    if not N.per[d] and (q[d] < 0 or q[d] > N.shape[d]):
                        continue
                    tot = 0.0
                    others = [e for e in range(dm) if e != d]
                    for bits in itertools.product((0, 1), repeat=dm - 1):
                        c = [0] * dm
                        c[d] = min(p[d], p[d] + s)
                        for e, b in zip(others, bits):
                            c[e] = p[e] - b
                        cc = N.cell(c)
                        tot += sigma[cc] if cc is not None else 0.0
                    se = tot / 2 ** (dm - 1) / N.dx[d] ** 2
                    rows.append(N.uid[p])
                    cols.append(N.uid[p])
                    vals.append(-se)
                    m = N.fold(tuple(q))
                    if m is not None:
                        rows.append(N.uid[p])
                        cols.append(N.uid[m])
                        vals.append(se)
    return sp.csr_matrix((vals, (rows, cols)), shape=(N.nunk, N.nunk))


def divu(N: Nodes, u, upad=None, inflow_lo=(0, 0, 0), inflow_hi=(0, 0, 0)):
    """Node-centred divergence (storage nodes), U = 0 outside non-periodic faces, except at an
    inflow face: there the ghost cell just outside (upad: U with one ghost layer, the inflow
    velocity on the wall) adds its normal component's flux through the face."""
    dm = N.dm
    out = np.zeros(N.nshape)
    for p in itertools.product(*[range(m) for m in N.nshape]):
        s = 0.0
        for a in itertools.product((0, 1), repeat=dm):
            raw = tuple(p[d] - a[d] for d in range(dm))
            cc = N.cell(raw)
            if cc is None:
                if upad is None:
                    continue
                # outside through exactly one inflow face (edges and corners carry nothing)
                out_dirs = [d for d in range(dm)
                            if not N.per[d] and (raw[d] < 0 or raw[d] >= N.shape[d])]
                if len(out_dirs) != 1:
                    continue
                d = out_dirs[0]
                if not (inflow_lo[d] if raw[d] < 0 else inflow_hi[d]):
                    continue
                g = tuple((raw[e] % N.shape[e] if N.per[e] else raw[e]) + 1 for e in range(dm))
                s += (-1.0 if a[d] else 1.0) * upad[g + (d,)] / N.dx[d]
                continue
            for d in range(dm):
                s += (-1.0 if a[d] else 1.0) * u[cc + (d,)] / N.dx[d]
        out[p] = s / 2 ** (dm - 1)
    return out


def grad(N: Nodes, phi):
    """mkgphi (Source/hgproject.f90:605-636)."""
    dm = N.dm
    g = np.zeros(N.shape + (dm,))
    for c in itertools.product(*[range(n) for n in N.shape]):
        for d in range(dm):
            s = 0.0
            for b in itertools.product((0, 1), repeat=dm):
                m = tuple((c[e] + b[e]) % N.shape[e] if N.per[e] else c[e] + b[e] for e in range(dm))
                s += (1.0 if b[d] else -1.0) * phi[m]
            g[c + (d,)] = s / 2 ** (dm - 1) / N.dx[d]
    return g


def to_storage(N: Nodes, x):
    phi = np.zeros(N.nshape)
    for p in itertools.product(*[range(m) for m in N.nshape]):
        q = N.fold(p)
        phi[p] = 0.0 if q is None else x[N.uid[q]]
    return phi


def solve(N: Nodes, sigma, rh, dense=True):
    A = operator(N, sigma, dense).tocsc()
    f = np.zeros(N.nunk)
    for p in itertools.product(*[range(m) for m in N.nshape]):
        if N.uid[p] >= 0:
            f[N.uid[p]] = rh[p]
    if not any(N.dlo) and not any(N.dhi):
        f = f - f.mean()
        one = np.ones((N.nunk, 1))
        B = sp.bmat([[A, sp.csr_matrix(one)], [sp.csr_matrix(one.T), None]]).tocsc()
        x = spl.spsolve(B, np.concatenate([f, [0.0]]))[:-1]
    else:
        x = spl.spsolve(A, f)
    return to_storage(N, x)


def reference_hgproject(unew, uold, gpi, rhohalf, pi, dx, bc_lo, bc_hi, proj_type, dt,
                        beta0=None, nodalrhs=None, dense=True, alt_energy_fix=False,
                        inflow=None):
    """Source/hgproject.f90:32-264 on one level, whole-domain arrays.

    inflow: dict(lo, hi, unew_pad, uold_pad, beta0_pad) -- inlet face flags and the fields with
    one ghost layer (beta0_pad None: beta0_cart without ghosts).  The ghost layer goes through
    create_uvec_for_projection as the reference's loops take it ((U - Uold) / dt on the first
    ghost layer for the pressure iterations, unchanged otherwise; walls and symmetry zeroed, which
    the divergence's U = 0 outside already is) and the beta0 scaling on beta0's ghost layer."""
    N = Nodes(rhohalf.shape, dx, bc_lo, bc_hi)
    dm = N.dm
    u = np.array(unew, dtype=np.float64)
    rho = np.array(rhohalf, dtype=np.float64)
    b0 = np.ones(rho.shape) if beta0 is None else np.asarray(beta0, dtype=np.float64)
    upad = None
    if inflow is not None:
        upad = np.array(inflow["unew_pad"], dtype=np.float64)
        if proj_type == HG_PRESSURE_ITERS:
            upad = (upad - inflow["uold_pad"]) / dt
        if inflow.get("beta0_pad") is not None:
            upad = upad * np.asarray(inflow["beta0_pad"])[..., None]
    if proj_type == HG_PRESSURE_ITERS:
        u = (u - uold) / dt
    elif proj_type == HG_REGULAR:
        u = u + dt * gpi / rho[..., None]
    alt = alt_energy_fix and proj_type not in (HG_INITIAL, HG_DIVU_ITERS)
    u = u * b0[..., None]
    rho = rho / b0
    if alt:
        rho = rho / b0
    if upad is None:
        rh = divu(N, u)
    else:
        rh = divu(N, u, upad, inflow["lo"], inflow["hi"])
    if nodalrhs is not None:
        rh = rh - nodalrhs
    phi = solve(N, 1.0 / rho, rh, dense)
    u = u / b0[..., None]
    rho = rho * b0
    if alt:
        rho = rho * b0
    g = grad(N, phi)
    if alt:
        g = g * b0[..., None]
    u = u - g / rho[..., None]
    gpi = np.array(gpi, dtype=np.float64)
    pi = np.array(pi, dtype=np.float64)
    if proj_type == HG_PRESSURE_ITERS:
        u = uold + dt * u
    if proj_type in (HG_INITIAL, HG_DIVU_ITERS):
        gpi[...] = 0.0
        pi[...] = 0.0
    elif proj_type == HG_PRESSURE_ITERS:
        gpi = gpi + g
        pi = pi + phi
    elif proj_type == HG_REGULAR:
        gpi = g / dt
        pi = phi / dt
    return u, gpi, pi, phi


def make_hg_case(shape, bc_lo, bc_hi, seed, with_beta0=True, with_rhs=True):
    """Seeded inputs: stratified density with noise, smooth-ish random velocities."""
    rng = np.random.default_rng(seed)
    dm = len(shape)
    z = (np.arange(shape[-1]) + 0.5) / shape[-1]
    sh = [1] * dm
    sh[-1] = shape[-1]
    rho0 = np.exp(-z / 0.3).reshape(sh)
    rho = rho0 * np.exp(0.05 * rng.standard_normal(shape))
    unew = rng.standard_normal(shape + (dm,))
    uold = rng.standard_normal(shape + (dm,))
    gpi = rng.standard_normal(shape + (dm,))
    pi = rng.standard_normal(tuple(n + 1 for n in shape))
    b0 = (rho0 ** (1 / 1.4)) * np.ones(shape) if with_beta0 else None
    nrhs = 0.1 * rng.standard_normal(tuple(n + 1 for n in shape)) if with_rhs else None
    return dict(unew=unew, uold=uold, gpi=gpi, rhohalf=rho, pi=pi, beta0=b0, nodalrhs=nrhs)


HG_CASES = {
    # 2-D dense, periodic x, walls in z, regular time step with beta0 and a nodal source
    "hg2d_32": dict(shape=(32, 32), bc=((BC_PER, BC_NEU), (BC_PER, BC_NEU)), proj=HG_REGULAR,
                    dense=True, alt=False, seed=11),
    # 2-D cross stencil, walls below / outflow above, the initial projection
    "hg2d_cross_outflow": dict(shape=(16, 24), bc=((BC_NEU, BC_NEU), (BC_NEU, BC_DIR)),
                               proj=HG_INITIAL, dense=False, alt=False, seed=12),
    # 3-D dense, periodic x/y, walls in z, pressure iterations with the alt energy fix
    "hg3d_12": dict(shape=(12, 12, 12), bc=((BC_PER, BC_PER, BC_NEU), (BC_PER, BC_PER, BC_NEU)),
                    proj=HG_PRESSURE_ITERS, dense=True, alt=True, seed=13),
}


# Inflow (inlet) faces: Neumann faces whose ghost cells carry the inflow velocity.
HG_INFLOW_CASES = {
    # 3-D dense, periodic x/y, inlet below / outflow above, regular time step; beta0_cart with a
    # ghost layer (the ghost velocity is scaled by it)
    "hg3d_inflow": dict(shape=(8, 8, 12), bc=((BC_PER, BC_PER, BC_NEU), (BC_PER, BC_PER, BC_DIR)),
                        proj=HG_REGULAR, dense=True, alt=False, seed=14, lo=(0, 0, 1), hi=(0, 0, 0),
                        b0_ghost=True),
    # 2-D dense, inlet on the left / outflow on the right, walls in y, pressure iterations with
    # the alt energy fix; beta0_cart without ghosts (the ghost velocity is not scaled)
    "hg2d_inflow_piters": dict(shape=(16, 12), bc=((BC_NEU, BC_NEU), (BC_DIR, BC_NEU)),
                               proj=HG_PRESSURE_ITERS, dense=True, alt=True, seed=15, lo=(1, 0, 0),
                               hi=(0, 0, 0), b0_ghost=False),
    # 2-D cross stencil, inlets on both y faces (no outflow: singular), the initial projection
    "hg2d_inflow_cross": dict(shape=(12, 16), bc=((BC_PER, BC_NEU), (BC_PER, BC_NEU)),
                              proj=HG_INITIAL, dense=False, alt=False, seed=16, lo=(0, 1, 0),
                              hi=(0, 1, 0), b0_ghost=True),
}


def build_inflow_case(name):
    """Inputs with one ghost layer: the valid region as make_hg_case draws it, ghost cells drawn
    independently (the caller's boundary fill)."""
    c = HG_INFLOW_CASES[name]
    shape = c["shape"]
    dm = len(shape)
    dx = tuple(1.0 / shape[0] for _ in shape)
    bc_lo, bc_hi = c["bc"]
    inp = make_hg_case(shape, bc_lo, bc_hi, c["seed"])
    rng = np.random.default_rng(c["seed"] + 100)
    pshape = tuple(n + 2 for n in shape)
    inner = tuple(slice(1, n + 1) for n in shape)
    upad = 0.5 + rng.standard_normal(pshape + (dm,))
    upad[inner] = inp["unew"]
    uopad = rng.standard_normal(pshape + (dm,))
    uopad[inner] = inp["uold"]
    bpad = None
    if c["b0_ghost"]:
        bpad = 1.0 + 0.2 * rng.random(pshape)
        bpad[inner] = inp["beta0"]
    inflow = dict(lo=c["lo"], hi=c["hi"], unew_pad=upad, uold_pad=uopad, beta0_pad=bpad)
    return c, shape, dx, bc_lo, bc_hi, inp, inflow


def build_case(name):
    c = HG_CASES[name]
    shape = c["shape"]
    dx = tuple(1.0 / shape[0] for _ in shape)
    bc_lo, bc_hi = c["bc"]
    inp = make_hg_case(shape, bc_lo, bc_hi, c["seed"])
    return c, shape, dx, bc_lo, bc_hi, inp


def main():
    for name in HG_CASES:
        c, shape, dx, bc_lo, bc_hi, inp = build_case(name)
        dt = 0.01
        u, gpi, pi, phi = reference_hgproject(inp["unew"], inp["uold"], inp["gpi"],
                                              inp["rhohalf"], inp["pi"], dx, bc_lo, bc_hi,
                                              c["proj"], dt, beta0=inp["beta0"],
                                              nodalrhs=inp["nodalrhs"], dense=c["dense"],
                                              alt_energy_fix=c["alt"])
        out = {k: v for k, v in inp.items() if v is not None}
        out.update(dx=np.array(dx), bc_lo=np.array(bc_lo), bc_hi=np.array(bc_hi),
                   proj=np.array(c["proj"]), dense=np.array(int(c["dense"])),
                   alt=np.array(int(c["alt"])), dt=np.array(dt), u_out=u, gpi_out=gpi,
                   pi_out=pi, phi_out=phi)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(path)
    for name in HG_INFLOW_CASES:
        c, shape, dx, bc_lo, bc_hi, inp, inflow = build_inflow_case(name)
        dt = 0.01
        u, gpi, pi, phi = reference_hgproject(inp["unew"], inp["uold"], inp["gpi"],
                                              inp["rhohalf"], inp["pi"], dx, bc_lo, bc_hi,
                                              c["proj"], dt, beta0=inp["beta0"],
                                              nodalrhs=inp["nodalrhs"], dense=c["dense"],
                                              alt_energy_fix=c["alt"], inflow=inflow)
        out = {k: v for k, v in inp.items() if v is not None}
        out.update(dx=np.array(dx), bc_lo=np.array(bc_lo), bc_hi=np.array(bc_hi),
                   proj=np.array(c["proj"]), dense=np.array(int(c["dense"])),
                   alt=np.array(int(c["alt"])), dt=np.array(dt), u_out=u, gpi_out=gpi,
                   pi_out=pi, phi_out=phi, inflow_lo=np.array(c["lo"]),
                   inflow_hi=np.array(c["hi"]), unew_pad=inflow["unew_pad"],
                   uold_pad=inflow["uold_pad"])
        if inflow["beta0_pad"] is not None:
            out["beta0_pad"] = inflow["beta0_pad"]
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(path)


if __name__ == "__main__":
    main()
