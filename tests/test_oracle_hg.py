"""The nodal (HG) projection oracle against its pins (no GPU).

Pins: the golden fixtures of tests/golden/make_golden_hg.py (an independent numpy/scipy assembly
of the nodal operators -- element stiffness by Gauss quadrature -- and a sparse direct solve), the
same script's operators, divergence and gradient applied live, and known answers: the constant
in the null space, symmetry, the closed 9-point form of the dense stencil, second-order
consistency with the Laplacian."""
import importlib.util
import os

import numpy as np
import pytest

import oracle as O
from maestro_gb300.inputs import BC_DIR, BC_NEU, BC_PER

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _gen():
    spec = importlib.util.spec_from_file_location("make_golden_hg",
                                                  os.path.join(GOLDEN, "make_golden_hg.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


G = _gen()


def load_hg(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["dx"] = tuple(float(v) for v in z["dx"])
    d["bc_lo"] = tuple(int(v) for v in z["bc_lo"])
    d["bc_hi"] = tuple(int(v) for v in z["bc_hi"])
    return d


def _unknown_mask(shape, dx, bc_lo, bc_hi):
    return G.Nodes(shape, dx, bc_lo, bc_hi).uid >= 0


@pytest.mark.parametrize("name", sorted(G.HG_CASES))
def test_oracle_hgproject_matches_golden(name):
    c = load_hg(name)
    shape = c["rhohalf"].shape
    u, gpi, pi, phi, st = O.hgproject(c["unew"], c["uold"], c["gpi"], c["rhohalf"], c["pi"],
                                      c["dx"], c["bc_lo"], c["bc_hi"], proj_type=int(c["proj"]),
                                      dt=float(c["dt"]), beta0_cart=c.get("beta0"),
                                      nodalrhs=c.get("nodalrhs"), dense=bool(c["dense"]),
                                      alt_energy_fix=bool(c["alt"]), rel_eps=1e-13)
    assert st["status"] == 0
    m = _unknown_mask(shape, c["dx"], c["bc_lo"], c["bc_hi"])
    singular = BC_DIR not in c["bc_lo"] + c["bc_hi"]
    a, b = phi[m], c["phi_out"][m]
    if singular:
        a, b = a - a.mean(), b - b.mean()
    # solved to 1e-13; phi, U, gpi within 1e-9 of the direct solve
    assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(b))
    assert np.max(np.abs(u - c["u_out"])) <= 1e-9 * np.max(np.abs(c["u_out"]))
    den = max(np.max(np.abs(c["gpi_out"])), 1e-300)
    assert np.max(np.abs(gpi - c["gpi_out"])) <= 1e-9 * max(den, np.max(np.abs(c["gpi"])))


@pytest.mark.parametrize("dense", [True, False])
@pytest.mark.parametrize("shape,bc_lo,bc_hi", [
    ((12, 10), (BC_PER, BC_NEU), (BC_PER, BC_NEU)),
    ((8, 12), (BC_NEU, BC_DIR), (BC_DIR, BC_NEU)),
    ((6, 8, 6), (BC_PER, BC_NEU, BC_NEU), (BC_PER, BC_NEU, BC_DIR)),
])
def test_operator_divergence_gradient_match_assembly(dense, shape, bc_lo, bc_hi):
    rng = np.random.default_rng(5)
    dx = tuple(1.0 / (n + 3) for n in shape)       # anisotropic spacing
    N = G.Nodes(shape, dx, bc_lo, bc_hi)
    sigma = np.exp(rng.standard_normal(shape))
    x = rng.standard_normal(N.nunk)
    phi = G.to_storage(N, x)
    Lphi = O.hg_apply(sigma, phi, dx, bc_lo, bc_hi, dense=dense)
    A = G.operator(N, sigma, dense)
    ref = G.to_storage(N, A @ x)
    m = N.uid >= 0
    assert np.max(np.abs(Lphi[m] - ref[m])) <= 1e-12 * np.max(np.abs(ref[m]))
    # the assembled operator is symmetric; the constant lies in its null space when no face is
    # an outflow
    assert abs(A - A.T).max() <= 1e-12 * abs(A).max()
    if BC_DIR not in bc_lo + bc_hi:
        assert np.max(np.abs(A @ np.ones(N.nunk))) <= 1e-12 * abs(A).max()
    u = rng.standard_normal(tuple(shape) + (len(shape),))
    np.testing.assert_allclose(O.hg_divu(u, dx, bc_lo, bc_hi), G.divu(N, u), rtol=0, atol=1e-11)
    np.testing.assert_allclose(O.hg_grad(phi, dx, bc_lo, bc_hi), G.grad(N, phi), rtol=0,
                               atol=1e-11)


def test_dense_stencil_closed_form_and_consistency():
    # unit coefficient on a square grid: (L phi)_p = (sum of the 8 neighbours - 8 phi_p) / (3 h^2)
    n = 16
    h = 1.0 / n
    x = np.arange(n + 1) * h
    X, Y = np.meshgrid(x, x, indexing="ij")
    phi = np.cos(2 * np.pi * X) * np.cos(2 * np.pi * Y)
    per = (BC_PER, BC_PER)
    L = O.hg_apply(np.ones((n, n)), phi, (h, h), per, per, dense=True)
    core = phi[:n, :n]
    nb = sum(np.roll(np.roll(core, a, 0), b, 1) for a in (-1, 0, 1) for b in (-1, 0, 1)
             if (a, b) != (0, 0))
    np.testing.assert_allclose(L[:n, :n], (nb - 8 * core) / (3 * h * h), rtol=0, atol=1e-9)
    # second-order consistency with div grad: the error drops ~4x per halving of h
    errs = []
    for m in (16, 32, 64):
        hh = 1.0 / m
        xx = np.arange(m + 1) * hh
        XX, YY = np.meshgrid(xx, xx, indexing="ij")
        f = np.cos(2 * np.pi * XX) * np.cos(2 * np.pi * YY)
        Lf = O.hg_apply(np.ones((m, m)), f, (hh, hh), per, per, dense=True)
        errs.append(np.max(np.abs(Lf[:m, :m] + 8 * np.pi ** 2 * f[:m, :m])))
    assert 3.5 < errs[0] / errs[1] < 4.5 and 3.5 < errs[1] / errs[2] < 4.5


@pytest.mark.parametrize("dense", [True, False])
def test_solve_reaches_maestro_tolerance_and_matches_direct_solve(dense):
    rng = np.random.default_rng(9)
    shape = (16, 16, 16)
    dx = (1 / 16,) * 3
    bc = (BC_PER, BC_PER, BC_NEU)
    sigma = np.exp(0.5 * rng.standard_normal(shape))
    rh = rng.standard_normal(O.node_shape(shape))
    phi, st = O.hg_solve(sigma, rh, dx, bc, bc, dense=dense)
    assert st["status"] == 0 and st["rel_resid"] <= O.EPS_HG
    N = G.Nodes(shape, dx, bc, bc)
    ref = G.solve(N, sigma, rh, dense)
    m = N.uid >= 0
    a, b = phi[m] - phi[m].mean(), ref[m] - ref[m].mean()
    assert np.max(np.abs(a - b)) <= 1e-8 * np.max(np.abs(b))


def load_inflow(name):
    c = load_hg(name)
    c["lo"] = tuple(int(v) for v in c["inflow_lo"])
    c["hi"] = tuple(int(v) for v in c["inflow_hi"])
    c["wall"] = O.hg_wall_from_ghosts(c["rhohalf"].shape, c["lo"], c["hi"], int(c["proj"]),
                                      float(c["dt"]), c["unew_pad"], c["uold_pad"],
                                      c.get("beta0_pad"))
    return c


def check_against_golden(c, u, gpi, pi, phi):
    """phi (mean-free when singular), U, gpi within 1e-9 of the direct solve; pi up to phi's
    constant."""
    shape = c["rhohalf"].shape
    m = _unknown_mask(shape, c["dx"], c["bc_lo"], c["bc_hi"])
    if phi is not None:
        a, b = phi[m], c["phi_out"][m]
        if BC_DIR not in c["bc_lo"] + c["bc_hi"]:
            a, b = a - a.mean(), b - b.mean()
        assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(b))
    assert np.max(np.abs(u - c["u_out"])) <= 1e-9 * np.max(np.abs(c["u_out"]))
    assert np.max(np.abs(gpi - c["gpi_out"])) <= 1e-9 * max(np.max(np.abs(c["gpi_out"])),
                                                             np.max(np.abs(c["gpi"])))
    assert np.ptp((pi - c["pi_out"])[m]) <= 1e-9 * max(np.max(np.abs(c["pi_out"])), 1.0)


@pytest.mark.parametrize("name", sorted(G.HG_INFLOW_CASES))
def test_oracle_hgproject_inflow_matches_golden(name):
    c = load_inflow(name)
    kw = dict(proj_type=int(c["proj"]), dt=float(c["dt"]), beta0_cart=c.get("beta0"),
              nodalrhs=c.get("nodalrhs"), dense=bool(c["dense"]),
              alt_energy_fix=bool(c["alt"]), rel_eps=1e-13)
    args = (c["unew"], c["uold"], c["gpi"], c["rhohalf"], c["pi"], c["dx"], c["bc_lo"],
            c["bc_hi"])
    u, gpi, pi, phi, st = O.hgproject(*args, inflow_lo=c["lo"], inflow_hi=c["hi"],
                                      wall=c["wall"], **kw)
    assert st["status"] == 0
    check_against_golden(c, u, gpi, pi, phi)
    # the inlets matter: without them U is far from the golden one
    u0, _, _, _, _ = O.hgproject(*args, **kw)
    assert np.max(np.abs(u0 - c["u_out"])) > 1e-3 * np.max(np.abs(c["u_out"]))


@pytest.mark.parametrize("shape,bc_lo,bc_hi,lo,hi", [
    ((6, 8, 5), (BC_PER, BC_NEU, BC_NEU), (BC_PER, BC_NEU, BC_DIR), (0, 1, 1), (0, 1, 0)),
    ((7, 6), (BC_NEU, BC_NEU), (BC_NEU, BC_DIR), (1, 1), (1, 0)),
])
def test_inflow_divergence_matches_assembly(shape, bc_lo, bc_hi, lo, hi):
    # the oracle's inflow divergence (via a projection's right-hand side: L phi = DU) against
    # the fixture script's ghost-cell divergence, anisotropic spacing, several inlets at once
    rng = np.random.default_rng(9)
    dm = len(shape)
    dx = tuple(1.0 / (n + 2) for n in shape)
    upad = rng.standard_normal(tuple(n + 2 for n in shape) + (dm,))
    inner = tuple(slice(1, n + 1) for n in shape)
    u = upad[inner]
    N = G.Nodes(shape, dx, bc_lo, bc_hi)
    ref = G.divu(N, u, upad, lo, hi)
    wall = O.hg_wall_from_ghosts(shape, lo, hi, O.HG_INITIAL, 1.0, upad)
    # the divergence of the initial projection is L phi on the unknown nodes
    rho = np.ones(shape)
    _, _, _, phi, st = O.hgproject(u, u, np.zeros_like(u), rho, np.zeros(N.nshape), dx, bc_lo,
                                   bc_hi, proj_type=O.HG_INITIAL, dense=True, rel_eps=1e-13,
                                   inflow_lo=lo, inflow_hi=hi, wall=wall)
    assert st["status"] == 0
    Lphi = O.hg_apply(1.0 / rho, phi, dx, bc_lo, bc_hi, dense=True)
    m = N.uid >= 0
    r = ref[m]
    if BC_DIR not in bc_lo + bc_hi:
        r = r - r.mean()
    assert np.max(np.abs(Lphi[m] - r)) <= 1e-10 * np.max(np.abs(r))
