"""The oracle's spherical form of the projection (beta0 given on every face, the
beta0_cart_edge multifab of Source/macproject.f90:155-161, 194-201, 236-241):

* fed with faces that carry the planar 1-D beta0 (beta0(k) on x/y faces, beta0_edge(k) on z
  faces) it is the planar projection (to rounding; the oracle's OpenMP reductions are not
  bitwise repeatable);
* on a star-like case (beta0 and rho depending on the distance from the centre) with outflow
  (Dirichlet) or periodic boundaries, the projected field satisfies div(beta0 U) = macrhs to the
  solver tolerance relative to the divergence it started from.
"""
import numpy as np
import pytest

import oracle as O
from maestro_gb300.inputs import make_case, make_spherical_case
from tests._util import load_golden, phi_rel_err, u_rel_err


def _constraint(u, uin, b0c, dx, rhs):
    div = 0
    div0 = 0
    for d in range(3):
        div = div + np.diff(u[d] * b0c[d], axis=d) / dx[d]
        div0 = div0 + np.diff(uin[d] * b0c[d], axis=d) / dx[d]
    return float(np.abs(div - rhs).max() / np.abs(div0 - rhs).max())


def test_cart_form_with_planar_beta0_is_the_planar_projection():
    c = make_case(dm=3, n=(16, 16, 16), box=(8, 8, 8), kmax=3, seed=3)
    nl = O.nlevels_for_boxes([c.box])
    u1, p1, s1 = O.macproject(c.umac, c.phi0, c.rho, c.dx, c.bc_lo, c.bc_hi, macrhs=c.macrhs,
                              beta0=c.beta0, beta0_edge=c.beta0_edge, nlevels=nl, rel_eps=1e-12)
    b0c = []
    for d in range(3):
        shp = [16, 16, 16]
        shp[d] += 1
        src = c.beta0_edge if d == 2 else c.beta0
        b0c.append(np.asfortranarray(np.broadcast_to(src.reshape(1, 1, -1), shp).copy()))
    u2, p2, s2 = O.macproject_cart(c.umac, c.phi0, c.rho, c.dx, c.bc_lo, c.bc_hi, b0c,
                                   macrhs=c.macrhs, nlevels=nl, rel_eps=1e-12)
    assert s1["status"] == 0 and s2["status"] == 0
    assert u_rel_err(u1, u2) <= 1e-13 and phi_rel_err(p1, p2, True) <= 1e-13
    assert _constraint(u1, c.umac, b0c, c.dx, c.macrhs) <= 1e-11


@pytest.mark.parametrize("bc", ["outflow", "periodic"])
def test_cart_form_projects_onto_the_constraint(bc):
    c = make_spherical_case(n=(32, 32, 32), box=(16, 16, 16), bc=bc)
    u, p, st = O.macproject_cart(c.umac, c.phi0, c.rho, c.dx, c.bc_lo, c.bc_hi, c.b0c,
                                 macrhs=c.macrhs, nlevels=O.nlevels_for_boxes([c.box]))
    assert st["status"] == 0 and st["rel_resid"] <= 1e-10
    assert _constraint(u, c.umac, c.b0c, c.dx, c.macrhs) <= 1e-10
    # idempotent to the tolerance: projecting the projected field changes it little
    u2, _, _ = O.macproject_cart(u, p, c.rho, c.dx, c.bc_lo, c.bc_hi, c.b0c, macrhs=c.macrhs,
                                 nlevels=O.nlevels_for_boxes([c.box]))
    assert u_rel_err(u2, u) <= 1e-8


def test_cart_form_matches_the_direct_solve_fixture():
    # tests/golden/sph3d_16.npz: the spherical form solved by sparse LU (make_golden.py), no MG
    g = load_golden("sph3d_16")
    phi0 = np.zeros(g["rho"].shape, order="F")
    u, p, st = O.macproject_cart(g["umac"], phi0, g["rho"], g["dx"], g["bc_lo"], g["bc_hi"],
                                 g["b0c"], macrhs=g["macrhs"],
                                 nlevels=O.nlevels_for_boxes([g["box"]]), rel_eps=1e-12)
    assert st["status"] == 0
    assert phi_rel_err(p, g["phi"], False) <= 1e-9
    assert u_rel_err(u, g["unew"]) <= 1e-9
