"""The allocation-free small solve (mac_solve_small_noalloc) against the allocating multigrid
entry point (mac_multigrid) on the same inputs, two calls in a row.

mac_solve_small_noalloc serves callers that cannot allocate GPU memory: it keeps its work
vectors in one fixed array inside the library, so every call shares that array.  The second call
below uses different inputs, so stale contents left by the first call would show up as a wrong
answer.  Tolerance: the parity bar of the other GPU tests -- both solves reach a 1e-10 relative
residual and phi (mean removed, the problem is singular) agrees to 1e-9 relative.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from maestro_gb300 import capi
from maestro_gb300.inputs import make_case
from maestro_gb300.macproject import BcTower, Layout, MacProjector

pytestmark = pytest.mark.gpu


def problem(seed):
    c = make_case(dm=3, n=(16, 16, 16), box=(16, 16, 16), H_frac=0.15, kmax=3, seed=seed)
    beta = O.mac_coeffs(c.rho, c.dx, c.bc_lo, c.bc_hi, c.beta0, c.beta0_edge)
    rh = np.random.default_rng(seed).standard_normal(c.n)
    rh = np.asfortranarray(rh - rh.mean())
    return c, beta, rh


def via_mac_multigrid(c, beta, rh):
    lay = Layout.tiled(c.n, c.box)
    per = [b == capi.MAC_BC_PER for b in c.bc_lo]
    P = MacProjector(lay, c.dx, BcTower(c.bc_lo, c.bc_hi))
    try:
        fphi = lay.to_fabs(np.zeros(c.n), ng=1)
        st = P.mac_multigrid(lay.to_fabs(rh, ng=0), fphi,
                             [lay.to_fabs(beta[d], ng=1, face_dir=d, periodic=per) for d in range(3)],
                             ng_rh=0, strict=True)
    finally:
        P.close()
    return lay.from_fabs(fphi, ng=1), st


def via_noalloc(torch, c, beta, rh, stream):
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).transpose())).to(dev)  # noqa: E731
    d_rh = t(rh)
    d_phi = torch.zeros_like(d_rh)
    d_b = [t(b) for b in beta]
    n = (ctypes.c_int * 3)(*c.n)
    dx = (ctypes.c_double * 3)(*c.dx)
    lo = (ctypes.c_int * 3)(*c.bc_lo)
    hi = (ctypes.c_int * 3)(*c.bc_hi)
    st = capi.MacStats()
    rc = capi.lib().mac_solve_small_noalloc(
        3, n, dx, lo, hi, d_rh.data_ptr(), d_phi.data_ptr(), d_b[0].data_ptr(), d_b[1].data_ptr(),
        d_b[2].data_ptr(), None, 1e-10, 5000, stream, ctypes.byref(st))
    torch.cuda.synchronize()
    return rc, np.asfortranarray(d_phi.cpu().numpy().transpose()), st.as_dict()


def test_noalloc_matches_mac_multigrid_two_calls(cuda_lib):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (71, 72):   # two calls in a row, different inputs
        c, beta, rh = problem(seed)
        ref, st_ref = via_mac_multigrid(c, beta, rh)
        rc, phi, st = via_noalloc(torch, c, beta, rh, stream)
        assert rc == capi.MAC_OK, (rc, capi.strerror(rc), st)
        assert st["rel_resid"] <= 1e-10 and st_ref["rel_resid"] <= 1e-10
        err = np.max(np.abs((phi - phi.mean()) - (ref - ref.mean()))) / np.max(np.abs(ref - ref.mean()))
        assert err <= 1e-9, (seed, err)


def test_noalloc_rejects_levels_above_its_limit(cuda_lib):
    n = (ctypes.c_int * 3)(32, 32, 32)   # 32768 cells > MAC_NOALLOC_MAX_CELLS
    dx = (ctypes.c_double * 3)(1 / 32, 1 / 32, 1 / 32)
    bc = (ctypes.c_int * 3)(capi.MAC_BC_PER, capi.MAC_BC_PER, capi.MAC_BC_NEU)
    st = capi.MacStats()
    rc = capi.lib().mac_solve_small_noalloc(3, n, dx, bc, bc, 8, 8, 8, 8, 8, None, 1e-10, 10,
                                            None, ctypes.byref(st))
    assert rc == capi.MAC_ERR_TOO_LARGE
