"""Failure handling of the CUDA path.  Faults are injected on the host (bad inputs, iteration
limits); every call must return its status code and leave the GPU usable."""
import numpy as np
import pytest

from maestro_gb300 import capi
from maestro_gb300.capi import MacError
from maestro_gb300.inputs import make_case
from maestro_gb300.macproject import BcTower, macproject

pytestmark = pytest.mark.gpu


def small():
    return make_case(dm=3, n=(16, 16, 16), box=(8, 8, 8), kmax=3, seed=41)


def run(c, **kw):
    return macproject(c.umac, c.phi0, c.rho, c.dx, BcTower(c.bc_lo, c.bc_hi), macrhs=c.macrhs,
                      beta0_1d=c.beta0, beta0_1d_edge=c.beta0_edge, box=c.box, **kw)


def test_nan_density_rejected(cuda_lib):
    c = small()
    c.rho[3, 4, 5] = np.nan
    with pytest.raises(MacError) as e:
        run(c)
    assert e.value.code == capi.MAC_ERR_BAD_DENSITY


def test_nonpositive_density_rejected(cuda_lib):
    c = small()
    c.rho[0, 0, 0] = -1.0
    with pytest.raises(MacError) as e:
        run(c)
    assert e.value.code == capi.MAC_ERR_BAD_DENSITY


def test_nan_velocity_rejected(cuda_lib):
    c = small()
    c.umac[1][2, 2, 2] = np.inf
    with pytest.raises(MacError) as e:
        run(c)
    assert e.value.code == capi.MAC_ERR_NONFINITE


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_iteration_limit_reports_not_converged(cuda_lib, precision):
    c = small()
    u, phi, st = run(c, precision=precision, max_vcycles=1)
    assert st["status"] == capi.MAC_ERR_NOT_CONVERGED
    if precision == "fp64":
        assert st["vcycles"] == 1
    else:   # one refinement step of inner_vcycles FP32 V-cycles
        assert st["refine_iters"] == 1 and st["vcycles"] == capi.default_opts().inner_vcycles
    assert st["rel_resid"] > 1e-10


def test_gpu_healthy_after_errors(cuda_lib):
    c = small()
    u, phi, st = run(c)
    assert st["status"] == 0 and st["rel_resid"] <= 1e-10


def test_zero_rhs_gives_zero_phi(cuda_lib):
    c = small()
    for u in c.umac:
        u[...] = 0.0
    c.macrhs[...] = 0.0
    u, phi, st = run(c)
    assert st["status"] == 0 and np.all(phi == 0.0)


def test_wait_expiry_reports_device_timeout_and_context_recovers(cuda_lib):
    """Fault injection on the staged finest-level kernels of the mixed-precision solve (64^3: the
    staged half-sweep and restriction run): with inject_wait_expiry the first wait of each block
    targets a barrier that no copy ever completes, so it gives up after wait_limit_s (1 ms here),
    the block drains its own copies and leaves, and the call returns MAC_ERR_DEVICE_TIMEOUT.  The
    same context then solves normally, bitwise equal to a fresh context."""
    from maestro_gb300.macproject import Layout, MacProjector
    c = make_case(dm=3, n=(64, 64, 64), box=(32, 32, 32), kmax=4, seed=43)
    lay = Layout.tiled(c.n, c.box)
    per = [b == capi.MAC_BC_PER for b in c.bc_lo]

    def project(P, strict=True):
        fu = [lay.to_fabs(c.umac[d], ng=1, face_dir=d, periodic=per) for d in range(3)]
        fphi = lay.to_fabs(c.phi0, ng=1)
        st = P.macproject(fu, fphi, lay.to_fabs(c.rho, ng=1, periodic=per),
                          lay.to_fabs(c.macrhs, ng=0), c.beta0, c.beta0_edge, strict=strict)
        return lay.from_fabs(fphi, ng=1), [lay.from_fabs(fu[d], ng=1, face_dir=d) for d in range(3)], st

    P = MacProjector(lay, c.dx, BcTower(c.bc_lo, c.bc_hi), precision="mixed", wait_limit_s=1e-3,
                     inject_wait_expiry=1)
    try:
        with pytest.raises(MacError) as e:
            project(P)
        assert e.value.code == capi.MAC_ERR_DEVICE_TIMEOUT
        P.set_opts(inject_wait_expiry=0, wait_limit_s=1.0)
        phi, u, st = project(P)
        assert st["status"] == 0 and st["rel_resid"] <= 1e-10
    finally:
        P.close()
    Q = MacProjector(lay, c.dx, BcTower(c.bc_lo, c.bc_hi), precision="mixed")
    try:
        phi_f, u_f, st_f = project(Q)
    finally:
        Q.close()
    np.testing.assert_array_equal(phi, phi_f)
    for a, b in zip(u, u_f):
        np.testing.assert_array_equal(a, b)


def test_wait_limit_option_is_checked(cuda_lib):
    from maestro_gb300.macproject import Layout, MacProjector
    c = small()
    lay = Layout.tiled(c.n, c.box)
    for bad in (dict(wait_limit_s=0.0), dict(wait_limit_s=11.0), dict(inject_wait_expiry=2)):
        with pytest.raises(MacError) as e:
            MacProjector(lay, c.dx, BcTower(c.bc_lo, c.bc_hi), **bad)
        assert e.value.code == capi.MAC_ERR_INVALID
