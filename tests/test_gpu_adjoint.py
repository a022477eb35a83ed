"""Adjoint of the MAC projection (mac_macproject_adjoint_dense) against central finite
differences of the forward GPU projection and against a gradient assembled from the CPU oracle's
solve of the adjoint right-hand side.

Loss L = sum(w . U_proj) over every face entry, w ~ N(0,1).  Finite differences: step 1e-6
relative (U: 1e-6 max|U| v; 1/rho and beta0: 1e-6 x value x v), v ~ N(0,1), 32 seeded directions
per input; forward solves driven to 1e-13 so the solver tolerance stays far below the step.
Tolerance: |FD - <grad, dv>| <= 1e-6 max(|FD|, |<grad, dv>|).
"""
import numpy as np
import pytest

import oracle as O
from maestro_gb300 import capi
from maestro_gb300.inputs import cell_to_edge, make_case
from maestro_gb300.macproject import BcTower, Layout, MacProjector

pytestmark = pytest.mark.gpu

N_DIRS = 32
STEP = 1e-6
TOL = 1e-6


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


class Problem:
    def __init__(self, torch, precision="fp64", alt=False, seed=91, n=(24, 24, 24), box=(12, 12, 12)):
        self.torch = torch
        self.c = make_case(dm=3, n=n, box=box, H_frac=0.15, noise=0.02, kmax=4, seed=seed,
                           with_w=True)
        c = self.c
        self.dev = torch.device("cuda", 0)
        lay = Layout.tiled(c.n, c.box)
        self.P = MacProjector(lay, c.dx, BcTower(c.bc_lo, c.bc_hi), precision=precision,
                              rel_eps=1e-13, use_alt_energy_fix=int(alt),
                              stream=torch.cuda.current_stream().cuda_stream)

    def t(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(np.asarray(a).transpose())).to(self.dev)

    def back(self, x):
        return np.asfortranarray(x.cpu().numpy().transpose())

    def loss(self, umac, rho, beta0):
        c = self.c
        u = [self.t(a) for a in umac]
        phi = self.torch.zeros(tuple(reversed(c.n)), dtype=self.torch.float64, device=self.dev)
        b0 = self.torch.from_numpy(np.ascontiguousarray(beta0)).to(self.dev)
        b0e = self.torch.from_numpy(cell_to_edge(beta0)).to(self.dev)
        rho_d = self.t(rho)
        rhs = self.t(c.macrhs)
        st = self.P.macproject_dense(u[0].data_ptr(), u[1].data_ptr(), u[2].data_ptr(),
                                     phi.data_ptr(), rho_d.data_ptr(), rhs.data_ptr(),
                                     b0.data_ptr(), b0e.data_ptr(), strict=True)
        self.torch.cuda.synchronize()
        return sum(float(np.sum(self.back(u[d]) * c.w[d])) for d in range(3)), st

    def gradient(self):
        c = self.c
        tt = self.torch
        u = [self.t(a) for a in c.umac]
        w = [self.t(a) for a in c.w]
        du = [tt.zeros_like(x) for x in u]
        rho = self.t(c.rho)
        rhs = self.t(c.macrhs)
        b0 = tt.from_numpy(c.beta0).to(self.dev)
        b0e = tt.from_numpy(c.beta0_edge).to(self.dev)
        drinv = tt.zeros_like(rho)
        dmac = tt.zeros_like(rho)
        phi = tt.zeros_like(rho)
        db0 = tt.zeros_like(b0)
        st = self.P.adjoint_dense([x.data_ptr() for x in u], rho.data_ptr(), rhs.data_ptr(),
                                  b0.data_ptr(), b0e.data_ptr(), [x.data_ptr() for x in w],
                                  [x.data_ptr() for x in du], drinv.data_ptr(), db0.data_ptr(),
                                  dmac.data_ptr(), phi.data_ptr())
        tt.cuda.synchronize()
        return ([self.back(x) for x in du], self.back(drinv), db0.cpu().numpy(), self.back(dmac),
                self.back(phi), st)

    def close(self):
        self.P.close()


def check_fd(prob, grad_dot, perturb, n_dirs=N_DIRS, seed=5):
    rng = np.random.default_rng(seed)
    worst = 0.0
    for _ in range(n_dirs):
        args_p, args_m, expected = perturb(rng)
        lp, _ = prob.loss(*args_p)
        lm, _ = prob.loss(*args_m)
        fd = (lp - lm) / 2.0
        ad = grad_dot(expected)
        err = abs(fd - ad) / max(abs(fd), abs(ad), 1e-300)
        worst = max(worst, err)
    return worst


@pytest.mark.parametrize("alt", [False, True])
def test_adjoint_matches_finite_differences(torch, alt):
    prob = Problem(torch, alt=alt)
    c = prob.c
    try:
        du, drinv, db0, dmac, phi, st = prob.gradient()
        assert st["status"] == 0
        umax = max(np.max(np.abs(a)) for a in c.umac)

        def pert_u(rng):
            v = [rng.standard_normal(a.shape) * STEP * umax for a in c.umac]
            return ([a + b for a, b in zip(c.umac, v)], c.rho, c.beta0), \
                   ([a - b for a, b in zip(c.umac, v)], c.rho, c.beta0), v

        worst_u = check_fd(prob, lambda v: sum(float(np.sum(g * x)) for g, x in zip(du, v)), pert_u)

        sigma = 1.0 / c.rho

        def pert_s(rng):
            v = rng.standard_normal(c.rho.shape) * STEP * sigma
            return ([*c.umac], np.asfortranarray(1.0 / (sigma + v)), c.beta0), \
                   ([*c.umac], np.asfortranarray(1.0 / (sigma - v)), c.beta0), v

        worst_s = check_fd(prob, lambda v: float(np.sum(drinv * v)), pert_s, seed=6)

        def pert_b(rng):
            v = rng.standard_normal(c.beta0.shape) * STEP * c.beta0
            return ([*c.umac], c.rho, c.beta0 + v), ([*c.umac], c.rho, c.beta0 - v), v

        worst_b = check_fd(prob, lambda v: float(np.sum(db0 * v)), pert_b, seed=7)
    finally:
        prob.close()
    assert worst_u <= TOL, worst_u
    assert worst_s <= TOL, worst_s
    assert worst_b <= TOL, worst_b


def test_adjoint_against_oracle_solve(torch):
    """dL/dmacrhs = nu and dL/dU = w + beta0 (nu_hi - nu_lo)/dx with nu from the CPU oracle's MG
    solve of the adjoint right-hand side lambda = G^T(c w) (numpy)."""
    prob = Problem(torch, seed=93)
    c = prob.c
    try:
        du, drinv, db0, dmac, phi, st = prob.gradient()
    finally:
        prob.close()
    beta = O.mac_coeffs(c.rho, c.dx, c.bc_lo, c.bc_hi, c.beta0, c.beta0_edge)
    n = c.n
    lam = np.zeros(n)
    for d in range(3):
        va = 2
        shp = [1, 1, 1]
        bb = c.beta0_edge if d == va else c.beta0
        shp[va] = bb.size
        cf = beta[d] / bb.reshape(shp)        # c = beta_f / beta0_f
        cw = cf * c.w[d]
        if c.bc_lo[d] == O.BC_PER:
            sl0 = [slice(None)] * 3
            sl0[d] = slice(0, 1)
            sln = [slice(None)] * 3
            sln[d] = slice(n[d], n[d] + 1)
            tot = cw[tuple(sl0)] + cw[tuple(sln)]
            cw = cw.copy()
            cw[tuple(sl0)] = tot
            cw[tuple(sln)] = tot
        else:
            cw = cw.copy()
            for q in (0, n[d]):
                sl = [slice(None)] * 3
                sl[d] = slice(q, q + 1)
                cw[tuple(sl)] = 0.0
        lam += np.diff(cw, axis=d) / c.dx[d]
    mu, sto = O.mac_multigrid(np.asfortranarray(lam), np.zeros(n, order="F"), beta, c.dx, c.bc_lo,
                              c.bc_hi, nlevels=O.nlevels_for_boxes([c.box]), rel_eps=1e-13)
    nu = mu - mu.mean()
    assert np.max(np.abs(dmac - nu)) <= 1e-8 * np.max(np.abs(nu))
    for d in range(3):
        pad = [(0, 0)] * 3
        pad[d] = (1, 1)
        nup = np.pad(nu, pad)
        shp = [1, 1, 1]
        bb = c.beta0_edge if d == 2 else c.beta0
        shp[2] = bb.size
        ref = c.w[d] + bb.reshape(shp) * np.diff(nup, axis=d) / c.dx[d]
        assert np.max(np.abs(du[d] - ref)) <= 1e-8 * np.max(np.abs(ref))


def test_adjoint_mixed_precision_matches_fp64(torch):
    a = Problem(torch, precision="fp64", seed=95)
    b = Problem(torch, precision="mixed", seed=95)
    try:
        ga = a.gradient()
        gb = b.gradient()
    finally:
        a.close()
        b.close()
    for x, y in zip(ga[0], gb[0]):
        assert np.max(np.abs(x - y)) <= 1e-9 * np.max(np.abs(x))
    assert np.max(np.abs(ga[1] - gb[1])) <= 1e-8 * np.max(np.abs(ga[1]))
    assert np.max(np.abs(ga[2] - gb[2])) <= 1e-8 * np.max(np.abs(ga[2]))
