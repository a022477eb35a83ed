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
