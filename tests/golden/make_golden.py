"""Generate the golden fixtures that pin the MAC-projection oracle.

The reference (Fortran + the un-vendored FBoxLib multigrid) cannot be built in this environment and
its repository holds no numeric outputs for the MAC path (its regression benchmarks live off-repo),
so the fixtures come from an MG-independent computation of the same discrete problem:

  * face coefficients  beta_f = beta0_f^p * 2 / (rho_L + rho_R)       Source/macproject.f90:698-738
  * right-hand side    rh = -(div(beta0 U) - macrhs)                  Source/macproject.f90:385-398
  * operator           -div(beta_f grad phi), 7/5-point cross stencil, Neumann faces dropped,
                       periodic faces wrapped, Dirichlet faces with the linear ghost -phi_0
  * solve              sparse LU (scipy.sparse.linalg.spsolve) with the mean of phi pinned
                       to zero for the singular periodic/Neumann problem
  * correction         beta0 U -= beta_f G phi, then / beta0                 Source/macproject.f90:908-975

Every array of this file is written by numpy/scipy code that shares nothing with the C++ oracle
or the CUDA library.  Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from maestro_gb300.inputs import BC_DIR, BC_NEU, BC_PER, make_case, make_spherical_case  # noqa: E402


def face_coeffs(rho, beta0, beta0_edge, bc_lo, bc_hi, p):
    dm = rho.ndim
    va = dm - 1
    out = []
    for d in range(dm):
        n = rho.shape[d]
        # ghost density: periodic wrap or copy of the boundary cell
        lo_idx = np.arange(-1, n)
        hi_idx = np.arange(0, n + 1)
        if bc_lo[d] == BC_PER:
            lo_idx = lo_idx % n
            hi_idx = hi_idx % n
        else:
            lo_idx = np.clip(lo_idx, 0, n - 1)
            hi_idx = np.clip(hi_idx, 0, n - 1)
        rl = np.take(rho, lo_idx, axis=d)
        rr = np.take(rho, hi_idx, axis=d)
        b = 2.0 / (rl + rr)
        if beta0 is not None:
            shp = [1] * dm
            if d == va:
                shp[va] = n + 1
                bb = beta0_edge.reshape(shp)
            else:
                shp[va] = rho.shape[va]
                bb = beta0.reshape(shp)
            b = b * bb ** p
        out.append(np.asfortranarray(b))
    return out


def matrix(beta, dx, bc_lo, bc_hi, shape):
    dm = len(shape)
    N = int(np.prod(shape))
    idx = np.arange(N).reshape(shape, order="F")
    rows, cols, vals = [], [], []
    diag = np.zeros(shape)
    for d in range(dm):
        n = shape[d]
        ih2 = 1.0 / dx[d] ** 2
        b = beta[d]
        # interior faces 1..n-1 (between cells q-1 and q)
        for q in range(1, n):
            sl_f = [slice(None)] * dm
            sl_f[d] = q
            sl_a = [slice(None)] * dm
            sl_a[d] = q - 1
            sl_b = [slice(None)] * dm
            sl_b[d] = q
            w = b[tuple(sl_f)] * ih2
            ia, ib = idx[tuple(sl_a)].ravel(order="F"), idx[tuple(sl_b)].ravel(order="F")
            wf = w.ravel(order="F")
            rows += [ia, ib]
            cols += [ib, ia]
            vals += [-wf, -wf]
            diag[tuple(sl_a)] += w
            diag[tuple(sl_b)] += w
        # boundary faces
        for side, q, cell in ((0, 0, 0), (1, n, n - 1)):
            bc = bc_lo[d] if side == 0 else bc_hi[d]
            sl_f = [slice(None)] * dm
            sl_f[d] = q
            sl_c = [slice(None)] * dm
            sl_c[d] = cell
            w = b[tuple(sl_f)] * ih2
            if bc == BC_PER:
                if side == 0:   # couple cell 0 with cell n-1 once
                    sl_o = [slice(None)] * dm
                    sl_o[d] = n - 1
                    ia, ib = idx[tuple(sl_c)].ravel(order="F"), idx[tuple(sl_o)].ravel(order="F")
                    wf = w.ravel(order="F")
                    rows += [ia, ib]
                    cols += [ib, ia]
                    vals += [-wf, -wf]
                    diag[tuple(sl_c)] += w
                    diag[tuple(sl_o)] += w
            elif bc == BC_DIR:
                diag[tuple(sl_c)] += 2.0 * w
    rows.append(idx.ravel(order="F"))
    cols.append(idx.ravel(order="F"))
    vals.append(diag.ravel(order="F"))
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                         shape=(N, N))


def grad(phi, dx, bc_lo, bc_hi, d):
    n = phi.shape[d]
    shape = list(phi.shape)
    shape[d] += 1
    g = np.zeros(shape, order="F")
    sl = lambda q: tuple(slice(None) if e != d else q for e in range(phi.ndim))  # noqa: E731
    g[sl(slice(1, n))] = np.diff(phi, axis=d) / dx[d]
    if bc_lo[d] == BC_PER:
        w = (np.take(phi, [0], axis=d) - np.take(phi, [n - 1], axis=d)) / dx[d]
        g[sl(slice(0, 1))] = w
        g[sl(slice(n, n + 1))] = w
    else:
        if bc_lo[d] == BC_DIR:
            g[sl(slice(0, 1))] = 2.0 * np.take(phi, [0], axis=d) / dx[d]
        if bc_hi[d] == BC_DIR:
            g[sl(slice(n, n + 1))] = -2.0 * np.take(phi, [n - 1], axis=d) / dx[d]
    return g


def reference_projection(case, p=1):
    dm = case.dm
    va = dm - 1
    n = case.n
    beta = face_coeffs(case.rho, case.beta0, case.beta0_edge, case.bc_lo, case.bc_hi, p)
    bu = []
    for d in range(dm):
        shp = [1] * dm
        if d == va:
            shp[va] = n[va] + 1
            bb = case.beta0_edge.reshape(shp)
        else:
            shp[va] = n[va]
            bb = case.beta0.reshape(shp)
        bu.append((case.umac[d] * bb, bb))
    div = sum(np.diff(bu[d][0], axis=d) / case.dx[d] for d in range(dm))
    rh = -(div - case.macrhs)
    A = matrix(beta, case.dx, case.bc_lo, case.bc_hi, n)
    f = rh.ravel(order="F")
    N = f.size
    singular = all(b != BC_DIR for b in case.bc_lo + case.bc_hi)
    if singular:
        f = f - f.mean()
        one = sp.csr_matrix(np.ones((1, N)))
        Aaug = sp.bmat([[A, one.T], [one, None]]).tocsc()
        x = spl.spsolve(Aaug, np.concatenate([f, [0.0]]))[:N]
    else:
        x = spl.spsolve(A.tocsc(), f)
    phi = x.reshape(n, order="F")
    u_new = []
    for d in range(dm):
        g = grad(phi, case.dx, case.bc_lo, case.bc_hi, d)
        u_new.append(np.asfortranarray((bu[d][0] - beta[d] * g) / bu[d][1]))
    return phi, u_new, rh


def reference_projection_cart(case, p=1):
    """The spherical form: beta0 given on every face (case.b0c), Source/macproject.f90:155-161,
    194-201, 236-241; otherwise as reference_projection."""
    dm = case.dm
    n = case.n
    beta = face_coeffs(case.rho, None, None, case.bc_lo, case.bc_hi, p)
    beta = [np.asfortranarray(beta[d] * case.b0c[d] ** p) for d in range(dm)]
    bu = [case.umac[d] * case.b0c[d] for d in range(dm)]
    div = sum(np.diff(bu[d], axis=d) / case.dx[d] for d in range(dm))
    rh = -(div - case.macrhs)
    A = matrix(beta, case.dx, case.bc_lo, case.bc_hi, n)
    f = rh.ravel(order="F")
    N = f.size
    singular = all(b != BC_DIR for b in case.bc_lo + case.bc_hi)
    if singular:
        f = f - f.mean()
        one = sp.csr_matrix(np.ones((1, N)))
        Aaug = sp.bmat([[A, one.T], [one, None]]).tocsc()
        x = spl.spsolve(Aaug, np.concatenate([f, [0.0]]))[:N]
    else:
        x = spl.spsolve(A.tocsc(), f)
    phi = x.reshape(n, order="F")
    u_new = []
    for d in range(dm):
        g = grad(phi, case.dx, case.bc_lo, case.bc_hi, d)
        u_new.append(np.asfortranarray((bu[d] - beta[d] * g) / case.b0c[d]))
    return phi, u_new, rh


# spherical-form cases (beta0 on every face): name -> make_spherical_case kwargs
CART_CASES = {
    "sph3d_16": dict(n=(16, 16, 16), box=(8, 8, 8), bc="outflow", kmax=3, seed=16),
}


CASES = {
    # name: (make_case kwargs, BC override, beta0 exponent)
    "strat2d_32": (dict(dm=2, n=(32, 32), box=(32, 32), H_frac=0.25, noise=0.01,
                        noise_kind="linear", kmax=4, seed=11), None, 1),
    "strat3d_16": (dict(dm=3, n=(16, 16, 16), box=(8, 8, 8), H_frac=0.25, noise=0.01,
                        noise_kind="lognormal", kmax=4, seed=12), None, 1),
    "stiff3d_16": (dict(dm=3, n=(16, 16, 16), box=(8, 8, 8), H_frac=0.072, noise=0.05,
                        noise_kind="lognormal", kmax=4, seed=13), None, 1),
    "outlet2d_32x16": (dict(dm=2, n=(32, 16), box=(16, 16), H_frac=0.25, noise=0.01,
                            noise_kind="linear", kmax=3, seed=14),
                       ((BC_PER, BC_NEU), (BC_PER, BC_DIR)), 1),
    "altfix2d_32": (dict(dm=2, n=(32, 32), box=(16, 16), H_frac=0.15, noise=0.01,
                         noise_kind="linear", kmax=4, seed=15), None, 2),
}


def build_case(name):
    kw, bcs, p = CASES[name]
    c = make_case(name=name, **kw)
    if bcs is not None:
        c.bc_lo, c.bc_hi = tuple(bcs[0]), tuple(bcs[1])
    return c, p


def main():
    for name in CASES:
        c, p = build_case(name)
        phi, u_new, rh = reference_projection(c, p)
        arrs = dict(rho=c.rho, beta0=c.beta0, beta0_edge=c.beta0_edge, macrhs=c.macrhs,
                    phi=phi, rh=rh, bc_lo=np.array(c.bc_lo), bc_hi=np.array(c.bc_hi),
                    dx=np.array(c.dx), box=np.array(c.box), p=np.array(p))
        for d in range(c.dm):
            arrs[f"u{d}"] = c.umac[d]
            arrs[f"unew{d}"] = u_new[d]
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **arrs)
        print(path, os.path.getsize(path))
    for name, kw in CART_CASES.items():
        c = make_spherical_case(name=name, **kw)
        phi, u_new, rh = reference_projection_cart(c, 1)
        arrs = dict(rho=c.rho, macrhs=c.macrhs, phi=phi, rh=rh, bc_lo=np.array(c.bc_lo),
                    bc_hi=np.array(c.bc_hi), dx=np.array(c.dx), box=np.array(c.box),
                    p=np.array(1))
        for d in range(c.dm):
            arrs[f"u{d}"] = c.umac[d]
            arrs[f"unew{d}"] = u_new[d]
            arrs[f"b0c{d}"] = c.b0c[d]
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **arrs)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
