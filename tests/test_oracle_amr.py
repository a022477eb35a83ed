"""The multi-level (AMR) MAC-projection oracle against its pins (no GPU).

Pins: the golden fixtures of tests/golden/make_golden_amr.py (an MG-independent sparse direct
solve of the composite problem, written with numpy/scipy), the live composite operator of the same
script, the one-level oracle (a fine level covering the whole domain is the one-level problem at
the fine resolution) and the known-answer properties of a projection: the composite divergence
constraint, idempotence, constants in the null space, conservation."""
import importlib.util
import os

import numpy as np
import pytest

import oracle as O
from maestro_gb300.inputs import (AMR_CASES, BC_DIR, BC_NEU, BC_PER, amr_case, average_down,
                                  make_amr_case)

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _gen():
    spec = importlib.util.spec_from_file_location("make_golden_amr",
                                                  os.path.join(GOLDEN, "make_golden_amr.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


G = _gen()


def load_amr(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    dm = int(z["n0"].size)
    nlev = int(z["nlev"])
    boxes = [[]]
    for l in range(1, nlev):
        b = z[f"boxes{l}"]
        boxes.append([(tuple(int(v) for v in r[:dm]), tuple(int(v) for v in r[dm:])) for r in b])
    d = dict(dm=dm, nlev=nlev, boxes=boxes, n0=tuple(int(v) for v in z["n0"]),
             dx0=tuple(float(v) for v in z["dx0"]), bc_lo=tuple(int(v) for v in z["bc_lo"]),
             bc_hi=tuple(int(v) for v in z["bc_hi"]))
    for key in ("rho", "macrhs", "phi"):
        d[key] = [np.asfortranarray(z[f"{key}{l}"]) for l in range(nlev)]
    d["beta0"] = [z[f"beta0_{l}"] for l in range(nlev)]
    d["beta0_edge"] = [z[f"beta0e_{l}"] for l in range(nlev)]
    d["umac"] = [[np.asfortranarray(z[f"u{l}_{k}"]) for k in range(dm)] for l in range(nlev)]
    d["unew"] = [[np.asfortranarray(z[f"unew{l}_{k}"]) for k in range(dm)] for l in range(nlev)]
    return d


def composite_demean(H, phi):
    s = sum(phi[l][H.valid[l]].sum() * np.prod(H.h[l]) for l in range(H.L))
    v = sum(H.valid[l].sum() * np.prod(H.h[l]) for l in range(H.L))
    m = s / v
    return [np.where(H.inm[l], phi[l] - m, 0.0) for l in range(H.L)]


def phi_err(H, a, b):
    a = composite_demean(H, a)
    b = composite_demean(H, b)
    den = max(np.max(np.abs(b[l][H.inm[l]])) for l in range(H.L))
    return max(np.max(np.abs(a[l] - b[l])[H.inm[l]]) for l in range(H.L)) / den


def u_err(H, a, b):
    e = 0.0
    for l in range(H.L):
        for d in range(H.dm):
            m = G.face_member(H, l, d)
            e = max(e, np.max(np.abs(a[l][d] - b[l][d])[m]) / np.max(np.abs(b[l][d][m])))
    return e


def run_oracle(c, **kw):
    return O.macproject_ml(c["umac"], [np.zeros_like(p) for p in c["phi"]], c["rho"], c["dx0"],
                           c["bc_lo"], c["bc_hi"], c["boxes"], macrhs=c["macrhs"],
                           beta0=c["beta0"], beta0_edge=c["beta0_edge"], **kw)


@pytest.mark.parametrize("name", sorted(AMR_CASES))
def test_oracle_matches_golden_direct_solve(name):
    c = load_amr(name)
    H = G.Hierarchy(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"])
    u, phi, st = run_oracle(c, rel_eps=1e-12)
    assert st["status"] == 0 and st["rel_resid"] <= 1e-12
    # the composite system is solved to 1e-12; phi and U within 1e-9 of the exact solution
    assert phi_err(H, phi, c["phi"]) <= 1e-9
    assert u_err(H, u, c["unew"]) <= 1e-9


@pytest.mark.parametrize("name", sorted(AMR_CASES))
def test_default_tolerance_and_divergence_constraint(name):
    # MAESTRO's tolerance for nlevs levels, min(1e-10 * 10^(nlevs-1), 1e-8); after the projection
    # the composite divergence of beta0 U_proj equals macrhs up to that residual
    c = load_amr(name)
    H = G.Hierarchy(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"])
    eps = O.ml_rel_eps(c["nlev"])
    u, phi, st = run_oracle(c)
    assert st["status"] == 0 and st["rel_resid"] <= eps
    rh0 = G_rh(c, H, c["umac"])
    rh1 = G_rh(c, H, u)
    scale = max(np.max(np.abs(rh0[l][H.valid[l]])) for l in range(H.L))
    # singular problem: the composite mean of rh is not in the range and stays
    mean = 0.0
    if BC_DIR not in c["bc_lo"] + c["bc_hi"]:
        s = sum(rh0[l][H.valid[l]].sum() * np.prod(H.h[l]) for l in range(H.L))
        v = sum(H.valid[l].sum() * np.prod(H.h[l]) for l in range(H.L))
        mean = s / v
    worst = max(np.max(np.abs(rh1[l][H.valid[l]] - mean)) for l in range(H.L))
    assert worst <= 2 * eps * scale


def G_rh(c, H, u):
    """divumac of Source/macproject.f90:332-421 on every level (valid cells are what count)."""
    dm = H.dm
    uu = [[np.array(x, order="F") for x in u[l]] for l in range(H.L)]
    for l in range(H.L):
        for d in range(dm):
            uu[l][d] = uu[l][d] * G.beta0_face(_case_like(c), l, d, H.shape[l])
    for l in range(H.L - 1, 0, -1):
        G.edge_restrict(H, uu[l - 1], uu[l], l)
    out = []
    for l in range(H.L):
        dv = sum(np.diff(uu[l][d], axis=d) / H.h[l][d] for d in range(dm))
        out.append(np.where(H.inm[l], -(dv - c["macrhs"][l]), 0.0))
    return out


class _case_like:
    def __init__(self, c):
        self.dm = c["dm"]
        self.beta0 = c["beta0"]
        self.beta0_edge = c["beta0_edge"]


@pytest.mark.parametrize("name", ["amr2d_32", "amr2d_3lev"])
def test_projection_is_idempotent(name):
    c = load_amr(name)
    H = G.Hierarchy(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"])
    u1, _, _ = run_oracle(c, rel_eps=1e-12)
    c2 = dict(c)
    c2["umac"] = u1
    u2, phi2, st = run_oracle(c2, rel_eps=1e-12)
    assert u_err(H, u2, u1) <= 1e-10
    scale = max(np.max(np.abs(p)) for p in c["phi"])
    assert max(np.max(np.abs(p)) for p in phi2) <= 1e-9 * scale


def _random_layout(dm, bc, seed):
    rng = np.random.default_rng(seed)
    if dm == 2:
        n0 = (16, 16)
        boxes = [[], [((8, 4), (23, 19)), ((0, 24), (7, 31))]]
    else:
        n0 = (8, 8, 8)
        boxes = [[], [((4, 4, 4), (11, 11, 11))]]
    dx0 = tuple(1.0 / n0[0] for _ in n0)
    bc_lo = tuple([BC_PER] * (dm - 1) + [bc])
    H = G.Hierarchy(n0, dx0, bc_lo, bc_lo, boxes)
    rho_f = np.exp(0.3 * rng.standard_normal(H.shape[1]))
    rho = [average_down(rho_f), rho_f]
    beta = [G.face_coeffs(rho[l], None, None, bc_lo, bc_lo, 1) for l in range(2)]
    return H, n0, dx0, bc_lo, boxes, beta, rng


@pytest.mark.parametrize("dm,bc", [(2, BC_NEU), (2, BC_DIR), (3, BC_NEU)])
def test_composite_operator_matches_assembled_matrix(dm, bc):
    H, n0, dx0, bc_lo, boxes, beta, rng = _random_layout(dm, bc, 7)
    x = rng.standard_normal(H.nunk)
    phi = [np.asfortranarray((H.V[l] @ x).reshape(H.shape[l], order="F")) for l in range(H.L)]
    zero = [np.zeros(H.shape[l], order="F") for l in range(H.L)]
    res, _ = O.ml_residual(zero, phi, beta, dx0, bc_lo, bc_lo, boxes)
    A = G.composite_matrix(H, beta)
    ax = A @ x
    got = np.concatenate([(-res[l]).ravel(order="F")[np.flatnonzero(H.valid[l].ravel(order="F"))]
                          for l in range(H.L)])
    assert np.max(np.abs(got - ax)) <= 1e-12 * np.max(np.abs(ax))


@pytest.mark.parametrize("dm,bc", [(2, BC_DIR), (3, BC_NEU)])
def test_composite_solve_matches_direct_solve(dm, bc):
    H, n0, dx0, bc_lo, boxes, beta, rng = _random_layout(dm, bc, 11)
    rh = [np.asfortranarray(np.where(H.inm[l], rng.standard_normal(H.shape[l]), 0.0))
          for l in range(H.L)]
    zero = [np.zeros(H.shape[l], order="F") for l in range(H.L)]
    phi, st = O.ml_solve(rh, zero, beta, dx0, bc_lo, bc_lo, boxes, rel_eps=1e-12)
    assert st["status"] == 0
    ref = G.composite_solve(H, beta, rh)
    if bc == BC_DIR:
        den = max(np.max(np.abs(r)) for r in ref)
        assert max(np.max(np.abs(phi[l] - ref[l])[H.inm[l]]) for l in range(H.L)) <= 1e-9 * den
    else:
        assert phi_err(H, phi, ref) <= 1e-9


def test_constants_in_null_space_and_conservation():
    H, n0, dx0, bc_lo, boxes, beta, rng = _random_layout(2, BC_NEU, 3)
    zero = [np.zeros(H.shape[l], order="F") for l in range(H.L)]
    one = [np.asfortranarray(np.where(H.inm[l], 1.0, 0.0)) for l in range(H.L)]
    res, mx = O.ml_residual(zero, one, beta, dx0, bc_lo, bc_lo, boxes)
    A = G.composite_matrix(H, beta)
    assert mx <= 1e-12 * abs(A).max()
    # conservative composite operator: the volume-weighted sum of L phi vanishes
    x = rng.standard_normal(H.nunk)
    phi = [np.asfortranarray((H.V[l] @ x).reshape(H.shape[l], order="F")) for l in range(H.L)]
    res, _ = O.ml_residual(zero, phi, beta, dx0, bc_lo, bc_lo, boxes)
    tot = sum(res[l][H.valid[l]].sum() * np.prod(H.h[l]) for l in range(H.L))
    mag = sum(np.abs(res[l][H.valid[l]]).sum() * np.prod(H.h[l]) for l in range(H.L))
    assert abs(tot) <= 1e-12 * mag


def test_fine_level_covering_the_domain_is_the_one_level_problem():
    # a level 1 that covers the whole domain leaves no coarse-fine face: its result is the
    # one-level projection at the fine resolution
    case = make_amr_case(dm=2, n0=(16, 16), boxes=[[], [((0, 0), (31, 31))]], seed=5)
    u, phi, st = O.macproject_ml(case.umac, case.phi0, case.rho, case.dx0, case.bc_lo, case.bc_hi,
                                 case.boxes, macrhs=case.macrhs, beta0=case.beta0,
                                 beta0_edge=case.beta0_edge, rel_eps=1e-12)
    u1, phi1, st1 = O.macproject(case.umac[1], case.phi0[1], case.rho[1], case.dx(1), case.bc_lo,
                                 case.bc_hi, macrhs=case.macrhs[1], beta0=case.beta0[1],
                                 beta0_edge=case.beta0_edge[1], rel_eps=1e-12)
    a = phi[1] - phi[1].mean()
    b = phi1 - phi1.mean()
    assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(b))
    for d in range(2):
        assert np.max(np.abs(u[1][d] - u1[d])) <= 1e-9 * np.max(np.abs(u1[d]))
    # the coarse level holds the averages of the fine faces and cells
    np.testing.assert_allclose(phi[0], average_down(phi[1]), rtol=0, atol=1e-12 * np.abs(b).max())


def test_invalid_layouts_are_rejected():
    case = amr_case("amr2d_32")
    rh = [np.zeros(case.shape(l), order="F") for l in range(2)]
    beta = [[np.ones([s + (d == e) for e, s in enumerate(case.shape(l))]) for d in range(2)]
            for l in range(2)]
    for boxes in ([[], [((1, 8), (46, 39))]],           # odd lo: not aligned to the ratio
                  [[], [((16, 8), (48, 39))]],          # even hi
                  [[], [((16, 8), (70, 39))]]):         # outside the domain
        with pytest.raises(ValueError):
            O.ml_solve(rh, rh, beta, case.dx0, case.bc_lo, case.bc_hi, boxes)
    # three levels whose level 2 is not nested one coarse cell inside level 1
    rh3 = [np.zeros(case.shape(l), order="F") for l in range(3)]
    beta3 = [[np.ones([s + (d == e) for e, s in enumerate(case.shape(l))]) for d in range(2)]
             for l in range(3)]
    with pytest.raises(ValueError):
        O.ml_solve(rh3, rh3, beta3, case.dx0, case.bc_lo, case.bc_hi,
                   [[], [((16, 16), (47, 47))], [((32, 32), (63, 63))]])
