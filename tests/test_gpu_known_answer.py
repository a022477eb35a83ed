"""Known answers of MAESTRO's projection unit test (Exec/UNIT_TESTS/test_projection), through the
CUDA MAC projection (C ABI, per-box host fabs), FP64 and mixed precision.

The unit test projects a divergence-free edge velocity with a gradient added and checks that the
gradient is removed: test_projection.f90:221-261 (2-D field of Almgren, Bell and Szymczak 1996),
:264-344 (3-D curl field), :680-827 / :870-1050 (the added gradients: the discrete gradient of a
cosine potential on periodic domains, an analytic one, zero on the walls, with slip walls).
Restated here as analytic formulas; rho = 1 and no beta0 (varden.f90:396-411).

  * periodic: P(u0 + G phi) = P(u0) to solver tolerance (G phi is a discrete gradient), and
    P(u0) - u0 = O(dx^2) (u0 is divergence-free analytically, not discretely);
  * slip walls: the analytic gradient is removed to O(dx^2), and P(P(u)) = P(u).
"""
import numpy as np
import pytest

from maestro_gb300.inputs import BC_NEU, BC_PER
from maestro_gb300.macproject import BcTower, macproject
pytestmark = pytest.mark.gpu

PRECISIONS = ["fp64", "mixed"]


def _rel(ua, ub):
    """max |ua - ub| / max |ub| over all components (a component may vanish)."""
    return max(np.max(np.abs(a - b)) for a, b in zip(ua, ub)) / max(np.max(np.abs(b)) for b in ub)


def _project(u, bc, dx, precision, box=None):
    n = tuple(u[d].shape[d] - 1 for d in range(len(u)))
    rho = np.ones(n, order="F")
    out, _, st = macproject([np.asfortranarray(a) for a in u], np.zeros(n, order="F"), rho, dx,
                            BcTower(bc, bc), box=box, precision=precision, rel_eps=1e-12)
    assert st["status"] == 0 and st["rel_resid"] <= 1e-12
    return out


def _field_2d(n):
    """test_projection.f90:221-261: u = -sin^2(pi x) sin(2 pi y) on x faces, v = sin^2(pi y)
    sin(2 pi x) on y faces (zero normal velocity on the unit square's walls)."""
    dx = 1.0 / n
    c = (np.arange(n) + 0.5) * dx
    f = np.arange(n + 1) * dx
    X, Y = np.meshgrid(f, c, indexing="ij")
    u = -np.sin(np.pi * X) ** 2 * np.sin(2 * np.pi * Y)
    X, Y = np.meshgrid(c, f, indexing="ij")
    v = np.sin(np.pi * Y) ** 2 * np.sin(2 * np.pi * X)
    return [u, v], (dx, dx)


def _field_3d(n):
    """test_projection.f90:264-344: the curl of (sin4pi y sin2pi z, sin2pi x sin4pi z,
    sin4pi x sin2pi y) on the faces."""
    dx = 1.0 / n
    c = (np.arange(n) + 0.5) * dx
    f = np.arange(n + 1) * dx
    pi = np.pi
    X, Y, Z = np.meshgrid(f, c, c, indexing="ij")
    u = 2 * pi * np.sin(4 * pi * X) * np.cos(2 * pi * Y) - 4 * pi * np.sin(2 * pi * X) * np.cos(4 * pi * Z)
    X, Y, Z = np.meshgrid(c, f, c, indexing="ij")
    v = 2 * pi * np.sin(4 * pi * Y) * np.cos(2 * pi * Z) - 4 * pi * np.cos(4 * pi * X) * np.sin(2 * pi * Y)
    X, Y, Z = np.meshgrid(c, c, f, indexing="ij")
    w = 2 * pi * np.cos(2 * pi * X) * np.sin(4 * pi * Z) - 4 * pi * np.cos(4 * pi * Y) * np.sin(2 * pi * Z)
    return [u, v, w], (dx, dx, dx)


def _discrete_gradient(n, dm, amp):
    """The face gradient of phi = amp prod_d cos(2 pi x_d) at cell centres (ghosts included,
    periodic): test_projection.f90:700-760 (2-D, amp 0.1) and :930-1000 (3-D, amp 5)."""
    dx = 1.0 / n
    cg = (np.arange(-1, n + 1) + 0.5) * dx
    grids = np.meshgrid(*([cg] * dm), indexing="ij")
    ph = amp * np.prod([np.cos(2 * np.pi * g) for g in grids], axis=0)
    inner = [slice(1, -1)] * dm
    out = []
    for d in range(dm):
        hi = list(inner)
        lo = list(inner)
        hi[d] = slice(1, None)
        lo[d] = slice(None, -1)
        out.append((ph[tuple(hi)] - ph[tuple(lo)]) / dx)
    return out


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("dm,n", [(2, 64), (3, 32)])
def test_periodic_gradient_is_removed(dm, n, precision):
    u0, dx = _field_2d(n) if dm == 2 else _field_3d(n)
    g = _discrete_gradient(n, dm, 0.1 if dm == 2 else 5.0)
    bc = (BC_PER,) * dm
    box = (n // 2,) * dm
    p_a = _project([a + b for a, b in zip(u0, g)], bc, dx, precision, box)
    p_b = _project(u0, bc, dx, precision, box)
    # P(u0 + G phi) = P(u0): the discrete gradient is removed to solver tolerance
    assert _rel(p_a, p_b) <= 1e-9
    # P(u0) - u0 = O(dx^2)
    assert _rel(p_b, u0) <= 50.0 / n ** 2


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("dm,n", [(2, 64), (3, 32)])
def test_wall_gradient_is_removed_and_projection_is_idempotent(dm, n, precision):
    u0, dx = _field_2d(n) if dm == 2 else _field_3d(n)
    if dm == 3:
        # a divergence-free field with zero normal velocity on the walls (this test's own: the
        # 3-D curl field's normal components do not vanish there): the 2-D field in x-y times
        # sin(pi z), no z component
        dxs = 1.0 / n
        c = (np.arange(n) + 0.5) * dxs
        f = np.arange(n + 1) * dxs
        X, Y, Z = np.meshgrid(f, c, c, indexing="ij")
        u = -np.sin(np.pi * X) ** 2 * np.sin(2 * np.pi * Y) * np.sin(np.pi * Z)
        X, Y, Z = np.meshgrid(c, f, c, indexing="ij")
        v = np.sin(np.pi * Y) ** 2 * np.sin(2 * np.pi * X) * np.sin(np.pi * Z)
        u0 = [u, v, np.zeros((n, n, n + 1))]
    # the analytic gradient 4 x (1 - x), ... (zero normal component on the walls):
    # test_projection.f90:703-722 (2-D), :870-915 (3-D, factor 160)
    amp = 4.0 if dm == 2 else 160.0
    dxs = 1.0 / n
    c = (np.arange(n) + 0.5) * dxs
    f = np.arange(n + 1) * dxs
    g = []
    for d in range(dm):
        axes = [c] * dm
        axes[d] = f
        X = np.meshgrid(*axes, indexing="ij")[d]
        g.append(amp * X * (1 - X))
    bc = (BC_NEU,) * dm
    box = (n // 2,) * dm
    p_u0 = _project(u0, bc, dx, precision, box)
    p_g = _project([a + b for a, b in zip(u0, g)], bc, dx, precision, box)
    # the analytic gradient is not a discrete one: removed to O(dx^2) of its size (amp / 4)
    err = max(np.max(np.abs(a - b)) for a, b in zip(p_g, p_u0))
    assert err <= (amp / 4.0) * 4.0 * dxs * dxs
    # idempotence
    p_pp = _project(p_g, bc, dx, precision, box)
    assert _rel(p_pp, p_g) <= 1e-9
