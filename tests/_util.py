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
