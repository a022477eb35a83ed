"""The CPU oracle against the golden fixtures and the known answers of MAESTRO's
test_projection unit test (CPU only)."""
import numpy as np
import pytest

import oracle as O
from tests._util import load_golden, phi_rel_err, rel_err, u_rel_err
from maestro_gb300.inputs import BC_DIR, BC_NEU, BC_PER, cell_to_edge, make_case

GOLDEN_CASES = ["strat2d_32", "strat3d_16", "stiff3d_16", "outlet2d_32x16", "altfix2d_32"]


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_direct_solve(name):
    g = load_golden(name)
    singular = all(b != BC_DIR for b in g["bc_lo"] + g["bc_hi"])
    nlev = O.nlevels_for_boxes([g["box"]])
    u, phi, st = O.macproject(g["umac"], np.zeros_like(g["rho"], order="F"), g["rho"], g["dx"],
                              g["bc_lo"], g["bc_hi"], macrhs=g["macrhs"], beta0=g["beta0"],
                              beta0_edge=g["beta0_edge"], nlevels=nlev, rel_eps=1e-12,
                              alt_energy_fix=g["p"] == 2)
    assert st["status"] == 0 and st["rel_resid"] <= 1e-12
    # both sides solve the same discrete system; tolerance 1e-9 relative (the parity bar)
    assert phi_rel_err(phi, g["phi"], singular) <= 1e-9
    assert u_rel_err(u, g["unew"]) <= 1e-9


def test_oracle_default_tolerance_and_level_count():
    g = load_golden("strat3d_16")
    nlev = O.nlevels_for_boxes([g["box"]])
    assert nlev == 3          # 8^3 boxes -> 8, 4, 2
    u, phi, st = O.macproject(g["umac"], np.zeros_like(g["rho"], order="F"), g["rho"], g["dx"],
                              g["bc_lo"], g["bc_hi"], macrhs=g["macrhs"], beta0=g["beta0"],
                              beta0_edge=g["beta0_edge"], nlevels=nlev)
    assert st["rel_resid"] <= 1e-10 and 3 <= st["vcycles"] <= 20
    # residual history decreases monotonically
    h = st["hist"]
    assert all(h[i + 1] < h[i] for i in range(len(h) - 1))


def test_nlevels_rule():
    assert O.nlevels_for_boxes([(128, 128, 128)]) == 7
    assert O.nlevels_for_boxes([(128, 128)]) == 7
    assert O.nlevels_for_boxes([(96, 96, 96)]) == 6   # 96 -> 48 -> 24 -> 12 -> 6 -> 3
    assert O.nlevels_for_boxes([(5, 5)]) == 1


def test_cell_to_edge_rule():
    b = np.exp(-np.linspace(0, 3, 17))
    e = O.cell_to_edge(b)
    assert e[0] == b[0] and e[-1] == b[-1]
    assert e[1] == 0.5 * (b[0] + b[1]) and e[-2] == 0.5 * (b[-1] + b[-2])
    tmp = 7 / 12 * (b[5] + b[4]) - 1 / 12 * (b[6] + b[3])
    assert e[5] == min(max(tmp, min(b[5], b[4])), max(b[5], b[4]))
    np.testing.assert_array_equal(e, cell_to_edge(b))


def _test_projection_periodic_3d(n):
    """Exec/UNIT_TESTS/test_projection: u0 = curl(sin4pi y sin2pi z, sin2pi x sin4pi z,
    sin4pi x sin2pi y) at faces (test_projection.f90:264-344) plus the discrete gradient of
    phi = 5 cos2pi x cos2pi y cos2pi z (:930-1000); rho = 1, no beta0 (varden.f90:396-411)."""
    dx = 1.0 / n
    c = (np.arange(n) + 0.5) * dx
    f = np.arange(n + 1) * dx
    pi = np.pi

    def grid(a, b, cc):
        return np.meshgrid(a, b, cc, indexing="ij")

    X, Y, Z = grid(f, c, c)
    u = 2 * pi * np.sin(4 * pi * X) * np.cos(2 * pi * Y) - 4 * pi * np.sin(2 * pi * X) * np.cos(4 * pi * Z)
    X, Y, Z = grid(c, f, c)
    v = 2 * pi * np.sin(4 * pi * Y) * np.cos(2 * pi * Z) - 4 * pi * np.cos(4 * pi * X) * np.sin(2 * pi * Y)
    X, Y, Z = grid(c, c, f)
    w = 2 * pi * np.cos(2 * pi * X) * np.sin(4 * pi * Z) - 4 * pi * np.cos(4 * pi * Y) * np.sin(2 * pi * Z)
    u0 = [np.asfortranarray(a) for a in (u, v, w)]
    cg = np.arange(-1, n + 1)
    X, Y, Z = grid((cg + 0.5) * dx, (cg + 0.5) * dx, (cg + 0.5) * dx)
    ph = 5.0 * np.cos(2 * pi * Y) * np.cos(2 * pi * X) * np.cos(2 * pi * Z)
    gx = (ph[1:, 1:-1, 1:-1] - ph[:-1, 1:-1, 1:-1]) / dx
    gy = (ph[1:-1, 1:, 1:-1] - ph[1:-1, :-1, 1:-1]) / dx
    gz = (ph[1:-1, 1:-1, 1:] - ph[1:-1, 1:-1, :-1]) / dx
    uin = [np.asfortranarray(a + g) for a, g in zip(u0, (gx, gy, gz))]
    return u0, uin, (dx, dx, dx)


def test_known_answer_periodic_projection():
    n = 32
    u0, uin, dx = _test_projection_periodic_3d(n)
    rho = np.ones((n, n, n), order="F")
    per = (BC_PER,) * 3
    u_a, _, st_a = O.macproject(uin, np.zeros_like(rho), rho, dx, per, per, rel_eps=1e-12)
    u_b, _, st_b = O.macproject(u0, np.zeros_like(rho), rho, dx, per, per, rel_eps=1e-12)
    # P(u0 + G phi) = P(u0): the discrete gradient is removed exactly (to solver tolerance)
    assert u_rel_err(u_a, u_b) <= 1e-9
    # P(u0) - u0 = O(dx^2): u0 is divergence-free analytically, not discretely
    assert u_rel_err(u_b, u0) <= 5.0 * (1.0 / n) ** 2 * 10


def test_known_answer_wall_projection():
    """Slip walls on all sides (inputs_3d_wall_mac): add 160 x(1-x) etc. (test_projection.f90:
    860-915) to a field with zero normal velocity on the walls; the projection removes it."""
    n = 16
    dx = 1.0 / n
    c = (np.arange(n) + 0.5) * dx
    f = np.arange(n + 1) * dx
    rng = np.random.default_rng(3)
    # a discretely divergence-free field with U.n = 0: the face curl of a random edge potential
    # would do; use the projection of random data instead
    neu = (BC_NEU,) * 3
    rho = np.ones((n, n, n), order="F")
    r = [rng.standard_normal((n + (d == 0), n + (d == 1), n + (d == 2))) for d in range(3)]
    for d in range(3):
        sl0 = [slice(None)] * 3
        sl0[d] = 0
        r[d][tuple(sl0)] = 0
        sl0[d] = n
        r[d][tuple(sl0)] = 0
    r = [np.asfortranarray(a) for a in r]
    u0, _, _ = O.macproject(r, np.zeros_like(rho), rho, (dx,) * 3, neu, neu, rel_eps=1e-13)
    X = np.meshgrid(f, c, c, indexing="ij")[0]
    Y = np.meshgrid(c, f, c, indexing="ij")[1]
    Z = np.meshgrid(c, c, f, indexing="ij")[2]
    g = [160 * X * (1 - X), 160 * Y * (1 - Y), 160 * Z * (1 - Z)]
    uin = [np.asfortranarray(a + b) for a, b in zip(u0, g)]
    u1, _, st = O.macproject(uin, np.zeros_like(rho), rho, (dx,) * 3, neu, neu, rel_eps=1e-13)
    # the analytic gradient is not a discrete gradient: recovered to O(dx^2) of its size (160/4)
    assert max(np.max(np.abs(a - b)) for a, b in zip(u1, u0)) <= 40.0 * 4 * dx * dx
    # idempotence of the projection
    u2, _, st2 = O.macproject(u1, np.zeros_like(rho), rho, (dx,) * 3, neu, neu, rel_eps=1e-13)
    assert u_rel_err(u2, u1) <= 1e-10


def test_divergence_constraint_after_projection():
    c = make_case(dm=3, n=(16, 16, 16), box=(8, 8, 8), kmax=4, seed=21)
    u, phi, st = O.macproject(c.umac, c.phi0, c.rho, c.dx, c.bc_lo, c.bc_hi, macrhs=c.macrhs,
                              beta0=c.beta0, beta0_edge=c.beta0_edge, nlevels=3)
    va = 2
    div = 0
    for d in range(3):
        shp = [1, 1, 1]
        bb = c.beta0_edge if d == va else c.beta0
        shp[va] = bb.size
        div = div + np.diff(u[d] * bb.reshape(shp), axis=d) / c.dx[d]
    # D(beta0 U_proj) = macrhs up to the solver tolerance (relative to the initial divergence)
    div0 = 0
    for d in range(3):
        shp = [1, 1, 1]
        bb = c.beta0_edge if d == va else c.beta0
        shp[va] = bb.size
        div0 = div0 + np.diff(c.umac[d] * bb.reshape(shp), axis=d) / c.dx[d]
    assert rel_err(div, c.macrhs + 0 * div) <= 2e-10 * np.max(np.abs(div0 - c.macrhs)) / np.max(np.abs(c.macrhs))


def _golden_module():
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "make_golden.py")
    spec = importlib.util.spec_from_file_location("make_golden", path)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize("bcs", ["wall", "outlet"])
def test_oracle_helmholtz_matches_direct_solve(bcs):
    # mac_multigrid with alpha != 0 (the thermal-diffusion form, Source/thermal_conduct.f90:375)
    # against a sparse LU solve of (alpha - div beta grad) phi = rh with the same discretisation
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    from maestro_gb300.inputs import BC_DIR, make_case
    g = _golden_module()
    c = make_case(dm=3, n=(16, 16, 16), box=(8, 8, 8), kmax=3, seed=21)
    if bcs == "outlet":
        c.bc_hi = (c.bc_hi[0], c.bc_hi[1], BC_DIR)
    beta = g.face_coeffs(c.rho, c.beta0, c.beta0_edge, c.bc_lo, c.bc_hi, 1)
    alpha = np.asfortranarray(c.rho * 1e-3)
    rh = np.asfortranarray(np.random.default_rng(4).standard_normal(c.n))
    A = g.matrix(beta, c.dx, c.bc_lo, c.bc_hi, c.n) + sp.diags(alpha.ravel(order="F"))
    x = spl.spsolve(A.tocsc(), rh.ravel(order="F")).reshape(c.n, order="F")
    phi, st = O.mac_multigrid(rh, np.zeros(c.n, order="F"), beta, c.dx, c.bc_lo, c.bc_hi,
                              alpha=alpha, nlevels=O.nlevels_for_boxes([c.box]), rel_eps=1e-12)
    assert st["status"] == 0
    assert rel_err(phi, x) <= 1e-9
