"""Shared helpers of the test suite (tolerances are stated where they are used)."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    dm = z["rho"].ndim
    d = {k: z[k] for k in z.files}
    d["dm"] = dm
    d["umac"] = [np.asfortranarray(z[f"u{i}"]) for i in range(dm)]
    d["unew"] = [np.asfortranarray(z[f"unew{i}"]) for i in range(dm)]
    d["bc_lo"] = tuple(int(v) for v in z["bc_lo"])
    d["bc_hi"] = tuple(int(v) for v in z["bc_hi"])
    d["dx"] = tuple(float(v) for v in z["dx"])
    d["box"] = tuple(int(v) for v in z["box"])
    d["p"] = int(z["p"])
    if "b0c0" in z.files:   # spherical form: beta0 on every face
        d["b0c"] = [np.asfortranarray(z[f"b0c{i}"]) for i in range(dm)]
    return d


def demean(a):
    return a - a.mean()


def rel_err(a, b):
    """max|a - b| / max|b|."""
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


def phi_rel_err(a, b, singular=True):
    if singular:
        return rel_err(demean(a), demean(b))
    return rel_err(a, b)


def u_rel_err(ua, ub):
    return max(rel_err(x, y) for x, y in zip(ua, ub))


def adjoint_reference(c, beta, rel_eps=1e-13, threads=0):
    """The oracle's gradient of L = sum(w . U_proj) (no beta0 derivative): nu, the mean-free
    solution of L mu = lambda with lambda = G^T(c w) (c = beta_f / beta0_f, walls excluded, the
    two copies of a periodic face summed), solved by the oracle's FP64 multigrid, and
    dL/dU_d = w_d + beta0_f (nu_hi - nu_lo) / dx_d (nu zero outside the domain).
    Returns (nu, [dU_d], stats)."""
    import oracle as O
    n = c.n
    dm = len(n)
    va = dm - 1
    lam = np.zeros(n)
    for d in range(dm):
        shp = [1] * dm
        bb = c.beta0_edge if d == va else c.beta0
        shp[va] = bb.size
        cw = beta[d] / bb.reshape(shp) * c.w[d]
        lo = [slice(None)] * dm
        lo[d] = slice(0, 1)
        hi = [slice(None)] * dm
        hi[d] = slice(n[d], n[d] + 1)
        if c.bc_lo[d] == O.BC_PER:
            tot = cw[tuple(lo)] + cw[tuple(hi)]
            cw[tuple(lo)] = tot
            cw[tuple(hi)] = tot
        else:
            cw[tuple(lo)] = 0.0
            cw[tuple(hi)] = 0.0
        lam += np.diff(cw, axis=d) / c.dx[d]
        del cw
    mu, st = O.mac_multigrid(np.asfortranarray(lam), np.zeros(n, order="F"), beta, c.dx, c.bc_lo,
                             c.bc_hi, nlevels=O.nlevels_for_boxes([c.box]), rel_eps=rel_eps,
                             threads=threads)
    del lam
    nu = mu - mu.mean()
    du = []
    for d in range(dm):
        pad = [(0, 0)] * dm
        pad[d] = (1, 1)
        shp = [1] * dm
        bb = c.beta0_edge if d == va else c.beta0
        shp[va] = bb.size
        du.append(c.w[d] + bb.reshape(shp) * np.diff(np.pad(nu, pad), axis=d) / c.dx[d])
    return nu, du, st
