"""The allocation-free small solve (mac_solve_small_noalloc) against the allocating multigrid
entry point (mac_multigrid) and against the CPU oracle's mac_multigrid, two calls in a row.

mac_solve_small_noalloc serves callers that cannot allocate GPU memory -- a host code whose
device memory all belongs to its own pool allocator, or a call site where cudaMalloc is not
allowed: it keeps its work vectors in one fixed array inside the library, so every call shares
that array.  The second call of each case uses different inputs, so stale contents left by the
first call would show up as a wrong answer.  Tolerance: the parity bar of the other GPU tests --
every solve reaches a 1e-10 relative residual, and phi (mean removed where the problem is
singular) agrees to 1e-9 relative.  This file is collected last, so a run that stops at its
first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from maestro_gb300 import capi
from maestro_gb300.inputs import make_case
from maestro_gb300.macproject import BcTower, Layout, MacProjector

pytestmark = pytest.mark.gpu

PER, NEU, DIR = capi.MAC_BC_PER, capi.MAC_BC_NEU, capi.MAC_BC_DIR

# name -> (dm, n, bc_lo, bc_hi, with alpha)
CASES = {
    "3d_per_neu": (3, (16, 16, 16), (PER, PER, NEU), (PER, PER, NEU), False),
    "2d_per_neu": (2, (64, 32), (PER, NEU), (PER, NEU), False),
    "3d_alpha_dir": (3, (16, 8, 16), (PER, NEU, NEU), (PER, NEU, DIR), True),
}


def problem(name, seed):
    dm, n, lo, hi, with_alpha = CASES[name]
    c = make_case(dm=dm, n=n, box=n, H_frac=0.15, kmax=3, seed=seed)
    beta = O.mac_coeffs(c.rho, c.dx, lo, hi, c.beta0, c.beta0_edge)
    rng = np.random.default_rng(seed)
    rh = rng.standard_normal(n)
    singular = not with_alpha and DIR not in lo and DIR not in hi
    if singular:
        rh -= rh.mean()
    alpha = None
    if with_alpha:
        # Helmholtz term of the size of the operator's diagonal (thermal diffusion's alpha = rho)
        alpha = np.asfortranarray(np.abs(rng.standard_normal(n)) * np.max(beta[0]) / c.dx[0] ** 2)
    return dict(c=c, n=n, dm=dm, lo=lo, hi=hi, beta=beta, rh=np.asfortranarray(rh), alpha=alpha,
                singular=singular)


def via_mac_multigrid(p):
    c, n = p["c"], p["n"]
    lay = Layout.tiled(n, n)
    per = [b == PER for b in p["lo"]]
    P = MacProjector(lay, c.dx, BcTower(p["lo"], p["hi"]))
    try:
        fphi = lay.to_fabs(np.zeros(n), ng=1)
        fal = lay.to_fabs(p["alpha"], ng=1) if p["alpha"] is not None else None
        st = P.mac_multigrid(lay.to_fabs(p["rh"], ng=0), fphi,
                             [lay.to_fabs(p["beta"][d], ng=1, face_dir=d, periodic=per)
                              for d in range(p["dm"])],
                             solver_alpha=fal, ng_rh=0, strict=True)
    finally:
        P.close()
    return lay.from_fabs(fphi, ng=1), st


def via_oracle(p):
    phi, st = O.mac_multigrid(p["rh"], np.zeros(p["n"]), p["beta"], p["c"].dx, p["lo"], p["hi"],
                              alpha=p["alpha"], rel_eps=1e-10)
    return phi, st


def via_noalloc(torch, p, stream, rel_eps=1e-10, max_iter=5000):
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).transpose())).to(dev)  # noqa: E731
    dm, n = p["dm"], p["n"]
    d_rh = t(p["rh"])
    d_phi = torch.zeros_like(d_rh)
    d_b = [t(b) for b in p["beta"]]
    d_al = t(p["alpha"]) if p["alpha"] is not None else None
    nn = (ctypes.c_int * 3)(*(list(n) + [1] * (3 - dm)))
    dx = (ctypes.c_double * 3)(*(list(p["c"].dx) + [1.0] * (3 - dm)))
    lo = (ctypes.c_int * 3)(*(list(p["lo"]) + [NEU] * (3 - dm)))
    hi = (ctypes.c_int * 3)(*(list(p["hi"]) + [NEU] * (3 - dm)))
    st = capi.MacStats()
    rc = capi.lib().mac_solve_small_noalloc(
        dm, nn, dx, lo, hi, d_rh.data_ptr(), d_phi.data_ptr(), d_b[0].data_ptr(),
        d_b[1].data_ptr(), d_b[2].data_ptr() if dm == 3 else None,
        d_al.data_ptr() if d_al is not None else None, rel_eps, max_iter, stream,
        ctypes.byref(st))
    torch.cuda.synchronize()
    return rc, np.asfortranarray(d_phi.cpu().numpy().transpose()), st.as_dict()


def rel_err(a, b, singular):
    if singular:
        a, b = a - a.mean(), b - b.mean()
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("name", sorted(CASES))
def test_noalloc_matches_mac_multigrid_and_oracle_two_calls(cuda_lib, name):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (71, 72):   # two calls in a row, different inputs
        p = problem(name, seed)
        ref, st_ref = via_mac_multigrid(p)
        orc, st_orc = via_oracle(p)
        rc, phi, st = via_noalloc(torch, p, stream)
        assert rc == capi.MAC_OK, (rc, capi.strerror(rc), st)
        assert st["rel_resid"] <= 1e-10 and st_ref["rel_resid"] <= 1e-10
        assert st_orc["rel_resid"] <= 1e-10
        e_lib = rel_err(phi, ref, p["singular"])
        e_orc = rel_err(phi, orc, p["singular"])
        assert e_lib <= 1e-9 and e_orc <= 1e-9, (name, seed, e_lib, e_orc)


@pytest.mark.parametrize("where", ["rh_singular", "rh_nonsingular", "beta"])
def test_noalloc_nan_input_is_reported(cuda_lib, where):
    """A NaN in the right-hand side (singular or not) or in a face coefficient gives
    MAC_ERR_NONFINITE, and the next call on clean inputs still solves."""
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream().cuda_stream
    p = problem("3d_alpha_dir" if where == "rh_nonsingular" else "3d_per_neu", 73)
    if where == "beta":
        p["beta"] = [b.copy(order="F") for b in p["beta"]]
        p["beta"][1][3, 4, 5] = np.nan
    else:
        p["rh"] = p["rh"].copy(order="F")
        p["rh"][2, 3, 4] = np.nan
    rc, _, st = via_noalloc(torch, p, stream)
    assert rc == capi.MAC_ERR_NONFINITE, (where, rc, capi.strerror(rc), st)
    clean = problem("3d_per_neu", 74)
    rc, phi, st = via_noalloc(torch, clean, stream)
    assert rc == capi.MAC_OK and st["rel_resid"] <= 1e-10, (rc, st)
    assert np.all(np.isfinite(phi))


def test_noalloc_rejects_levels_above_its_limit(cuda_lib):
    n = (ctypes.c_int * 3)(32, 32, 32)   # 32768 cells > MAC_NOALLOC_MAX_CELLS
    dx = (ctypes.c_double * 3)(1 / 32, 1 / 32, 1 / 32)
    bc = (ctypes.c_int * 3)(PER, PER, NEU)
    st = capi.MacStats()
    rc = capi.lib().mac_solve_small_noalloc(3, n, dx, bc, bc, 8, 8, 8, 8, 8, None, 1e-10, 10,
                                            None, ctypes.byref(st))
    assert rc == capi.MAC_ERR_TOO_LARGE
