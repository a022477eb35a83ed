"""The fused red/black sweep of the finest FP32 level (one kernel a sweep, out of place) against
the two half-sweep kernels it replaces: the mixed-precision solve gives bitwise the same phi and
velocities with the same cycle counts (the per-cell arithmetic is the same, in the same order),
with over-relaxed and Gauss-Seidel inner cycles, an odd and an even number of post-smoothing
sweeps, periodic, wall and Dirichlet faces."""
import numpy as np
import pytest

from maestro_gb300.inputs import BC_DIR, BC_NEU, BC_PER, make_case
from maestro_gb300.macproject import BcTower, macproject

pytestmark = pytest.mark.gpu

CASES = {
    "strat64": (dict(dm=3, n=(64, 64, 64), box=(32, 32, 32), H_frac=0.25, kmax=6, seed=51), None),
    "outlet64": (dict(dm=3, n=(64, 64, 64), box=(32, 32, 32), H_frac=0.25, kmax=4, seed=52),
                 ((BC_PER, BC_PER, BC_NEU), (BC_PER, BC_PER, BC_DIR))),
    "walls64x32x64": (dict(dm=3, n=(64, 32, 64), box=(32, 32, 32), H_frac=0.15, kmax=4, seed=53),
                      ((BC_NEU, BC_PER, BC_NEU), (BC_NEU, BC_PER, BC_NEU))),
}
CYCLES = {"sor_v21": dict(), "gs_v22": dict(inner_omega=1.0, inner_nu2=2),
          "sor_v22": dict(inner_nu2=2)}


@pytest.mark.parametrize("cycle", sorted(CYCLES))
@pytest.mark.parametrize("name", sorted(CASES))
def test_fused_sweep_bitwise_equals_half_sweeps(cuda_lib, name, cycle):
    kw, bcs = CASES[name]
    c = make_case(name=name, **kw)
    if bcs:
        c.bc_lo, c.bc_hi = bcs
    out = []
    for fused in (1, 0):
        u, phi, st = macproject(c.umac, c.phi0, c.rho, c.dx, BcTower(c.bc_lo, c.bc_hi),
                                macrhs=c.macrhs, beta0_1d=c.beta0, beta0_1d_edge=c.beta0_edge,
                                box=c.box, precision="mixed", fused_sweep=fused, **CYCLES[cycle])
        assert st["status"] == 0 and st["rel_resid"] <= 1e-10, st
        out.append((u, phi, st))
    (u1, p1, s1), (u0, p0, s0) = out
    np.testing.assert_array_equal(p1, p0)
    for a, b in zip(u1, u0):
        np.testing.assert_array_equal(a, b)
    assert s1["vcycles"] == s0["vcycles"] and s1["refine_iters"] == s0["refine_iters"]
    assert s1["launches"] < s0["launches"]   # the fused path did run
