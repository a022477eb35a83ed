"""Spherical form of the MAC projection on the GPU (beta0 on every face,
mac_macproject_cart / mac_macproject_cart_dense) against the oracle's restatement of it:
star-like cases (rho and beta0 depending on the distance from the centre) with outflow
(Dirichlet) and periodic boundaries, FP64 and mixed precision, whole-domain device arrays and
per-box host fabs; fed with the planar beta0 it is the planar projection."""
import numpy as np
import pytest

import oracle as O
from maestro_gb300.inputs import BC_DIR, make_case, make_spherical_case
from maestro_gb300.macproject import BcTower, Layout, MacProjector, macproject, macproject_cart
from tests._util import load_golden, phi_rel_err, u_rel_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _oracle(c, **kw):
    return O.macproject_cart(c.umac, c.phi0, c.rho, c.dx, c.bc_lo, c.bc_hi, c.b0c,
                             macrhs=c.macrhs, nlevels=O.nlevels_for_boxes([c.box]), **kw)


def _dense(c, precision, **opts):
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).transpose())).to(dev)  # noqa: E731
    u = [t(a) for a in c.umac]
    b = [t(a) for a in c.b0c]
    phi, rho, rhs = t(c.phi0), t(c.rho), t(c.macrhs)
    P = MacProjector(Layout.tiled(c.n, c.box), c.dx, BcTower(c.bc_lo, c.bc_hi),
                     precision=precision, stream=torch.cuda.current_stream().cuda_stream, **opts)
    try:
        st = P.macproject_cart_dense(u[0].data_ptr(), u[1].data_ptr(), u[2].data_ptr(),
                                     phi.data_ptr(), rho.data_ptr(), b[0].data_ptr(),
                                     b[1].data_ptr(), b[2].data_ptr(), macrhs=rhs.data_ptr(),
                                     strict=True)
    finally:
        P.close()
    torch.cuda.synchronize()
    back = lambda x: np.asfortranarray(x.cpu().numpy().transpose())  # noqa: E731
    return [back(x) for x in u], back(phi), st


@pytest.mark.parametrize("bc", ["outflow", "periodic"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cart_dense_matches_oracle(cuda_lib, bc, precision):
    c = make_spherical_case(n=(32, 32, 32), box=(16, 16, 16), bc=bc, seed=11)
    u_o, phi_o, st_o = _oracle(c)
    u, phi, st = _dense(c, precision)
    assert st["status"] == 0 and st["rel_resid"] <= 1e-10
    tol = 1e-9   # FP64 and mixed alike
    singular = bc == "periodic"
    assert phi_rel_err(phi, phi_o, singular) <= tol
    assert u_rel_err(u, u_o) <= tol
    if precision == "fp64":
        assert abs(st["vcycles"] - st_o["vcycles"]) <= 1


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cart_box_api_host_fabs_matches_oracle(cuda_lib, precision):
    c = make_spherical_case(n=(32, 32, 32), box=(16, 16, 16), bc="outflow", seed=12)
    u_o, phi_o, _ = _oracle(c)
    u, phi, st = macproject_cart(c.umac, c.phi0, c.rho, c.dx, BcTower(c.bc_lo, c.bc_hi), c.b0c,
                                 macrhs=c.macrhs, box=c.box, precision=precision)
    assert st["status"] == 0 and st["rel_resid"] <= 1e-10
    tol = 1e-9   # FP64 and mixed alike
    assert phi_rel_err(phi, phi_o, False) <= tol
    assert u_rel_err(u, u_o) <= tol


def test_cart_alt_energy_fix_matches_oracle(cuda_lib):
    c = make_spherical_case(n=(32, 32, 32), box=(16, 16, 16), bc="outflow", seed=13)
    u_o, phi_o, _ = _oracle(c, alt_energy_fix=True)
    u, phi, st = _dense(c, "fp64", use_alt_energy_fix=1)
    assert st["status"] == 0
    assert phi_rel_err(phi, phi_o, False) <= 1e-9 and u_rel_err(u, u_o) <= 1e-9


def test_cart_with_planar_beta0_is_the_planar_projection(cuda_lib):
    c = make_case(dm=3, n=(32, 32, 32), box=(16, 16, 16), kmax=4, seed=14)
    c.bc_hi = (c.bc_hi[0], c.bc_hi[1], BC_DIR)
    b0c = []
    for d in range(3):
        shp = [32, 32, 32]
        shp[d] += 1
        src = c.beta0_edge if d == 2 else c.beta0
        b0c.append(np.asfortranarray(np.broadcast_to(src.reshape(1, 1, -1), shp).copy()))
    bc = BcTower(c.bc_lo, c.bc_hi)
    u1, p1, s1 = macproject(c.umac, c.phi0, c.rho, c.dx, bc, macrhs=c.macrhs, beta0_1d=c.beta0,
                            beta0_1d_edge=c.beta0_edge, box=c.box, rel_eps=1e-12)
    u2, p2, s2 = macproject_cart(c.umac, c.phi0, c.rho, c.dx, bc, b0c, macrhs=c.macrhs,
                                 box=c.box, rel_eps=1e-12)
    assert s1["status"] == 0 and s2["status"] == 0
    assert phi_rel_err(p1, p2, False) <= 1e-10 and u_rel_err(u1, u2) <= 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cart_matches_the_direct_solve_fixture(cuda_lib, precision):
    # tests/golden/sph3d_16.npz: the spherical form solved by sparse LU, no multigrid involved
    g = load_golden("sph3d_16")
    phi0 = np.zeros(g["rho"].shape, order="F")
    u, phi, st = macproject_cart(g["umac"], phi0, g["rho"], g["dx"],
                                 BcTower(g["bc_lo"], g["bc_hi"]), g["b0c"], macrhs=g["macrhs"],
                                 box=g["box"], precision=precision, rel_eps=1e-12)
    assert st["status"] == 0 and st["rel_resid"] <= 1e-12
    assert phi_rel_err(phi, g["phi"], False) <= 1e-9
    assert u_rel_err(u, g["unew"]) <= 1e-9
