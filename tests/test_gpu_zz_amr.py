"""Multi-level (AMR) MAC projection on the GPU (mac_ctx_set_amr + mac_macproject_ml_dense)
against the golden direct solves of the composite problem and the oracle: two and three levels,
fine boxes wrapping a periodic boundary and touching a wall, 2-D and 3-D.  The kernels' cell
arithmetic is the code tests/test_amr_host_exec.py runs on the host."""
import numpy as np
import pytest

import oracle as O
from maestro_gb300 import capi
from maestro_gb300.inputs import AMR_CASES
from maestro_gb300.macproject import BcTower, Layout, MacError, MacProjector
from tests.test_oracle_amr import G, load_amr, phi_err, u_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _run(c, strict=True, rho=None, boxes=None, precision="fp64", **opts):
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).transpose())).to(dev)  # noqa: E731
    nlev = c["nlev"]
    dm = c["dm"]
    u = [[t(x) for x in c["umac"][l]] for l in range(nlev)]
    phi = [t(np.zeros_like(p)) for p in c["phi"]]
    rh = [t(r) for r in (rho if rho is not None else c["rho"])]
    mr = [t(m) for m in c["macrhs"]]
    b0 = [t(b) for b in c["beta0"]]
    b0e = [t(b) for b in c["beta0_edge"]]
    P = MacProjector(Layout(c["n0"], [((0,) * dm, tuple(v - 1 for v in c["n0"]))]), c["dx0"],
                     BcTower(c["bc_lo"], c["bc_hi"]), precision=precision,
                     stream=torch.cuda.current_stream().cuda_stream, **opts)
    try:
        P.set_amr(boxes if boxes is not None else c["boxes"])
        st = P.macproject_ml_dense([[x.data_ptr() for x in u[l]] for l in range(nlev)],
                                   [p.data_ptr() for p in phi], [r.data_ptr() for r in rh],
                                   macrhs=[m.data_ptr() for m in mr],
                                   beta0=[b.data_ptr() for b in b0],
                                   beta0_edge=[b.data_ptr() for b in b0e], strict=strict)
    finally:
        P.close()
    torch.cuda.synchronize()
    back = lambda x: np.asfortranarray(x.cpu().numpy().transpose())  # noqa: E731
    return [[back(x) for x in u[l]] for l in range(nlev)], [back(p) for p in phi], st


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", sorted(AMR_CASES))
def test_amr_projection_matches_golden(name, precision):
    c = load_amr(name)
    H = G.Hierarchy(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"])
    # rel_eps 1e-13 -> the composite tolerance min(1e-13 * 10^(nlev-1), 1e-8); mixed: FP32
    # multi-level cycles under FP64 refinement, the same tolerance on the FP64 residual
    u, phi, st = _run(c, rel_eps=1e-13, precision=precision)
    assert st["status"] == 0 and st["rel_resid"] <= 1e-13 * 10 ** (c["nlev"] - 1)
    assert phi_err(H, phi, c["phi"]) <= 1e-9
    assert u_err(H, u, c["unew"]) <= 1e-9


@pytest.mark.parametrize("name", ["amr2d_3lev", "amr3d_16"])
def test_amr_projection_matches_oracle_at_maestro_tolerance(name):
    c = load_amr(name)
    H = G.Hierarchy(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"])
    eps = O.ml_rel_eps(c["nlev"])
    u, phi, st = _run(c)
    assert st["status"] == 0 and st["rel_resid"] <= eps
    uo, po, so = O.macproject_ml(c["umac"], [np.zeros_like(p) for p in c["phi"]], c["rho"],
                                 c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"],
                                 macrhs=c["macrhs"], beta0=c["beta0"],
                                 beta0_edge=c["beta0_edge"], rel_eps=eps)
    # both solve the same composite system to eps; their distance is bounded by the error of
    # each against the exact solution
    assert phi_err(H, phi, po) <= 1e-7
    assert u_err(H, u, uo) <= 1e-7
    assert phi_err(H, phi, c["phi"]) <= 1e-7


def test_amr_layout_and_density_errors():
    c = load_amr("amr2d_32")
    with pytest.raises(MacError) as e:
        _run(c, boxes=[[], [((1, 8), (46, 39))]])   # not aligned to the ratio
    assert e.value.code == capi.MAC_ERR_INVALID
    rho = [np.array(r) for r in c["rho"]]
    rho[1][20, 20] = -1.0                               # inside the fine box
    with pytest.raises(MacError) as e:
        _run(c, rho=rho)
    assert e.value.code == capi.MAC_ERR_BAD_DENSITY


@pytest.mark.parametrize("name", ["amr2d_32", "amr2d_outflow", "amr2d_wrap", "amr3d_16",
                                  "amr3d_3lev"])
def test_amr_projection_on_host_fabs(name):
    # the drop-in form: per-box host fabs of every level (several boxes on level 0 too), rho with
    # two ghost cells, umac with one (the fine levels' ghost faces filled as create_umac_grown
    # fills them)
    c = load_amr(name)
    H = G.Hierarchy(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"])
    dm = c["dm"]
    nlev = c["nlev"]
    per = [b == O.BC_PER for b in c["bc_lo"]]
    lays = [Layout.tiled(c["n0"], tuple(v // 2 for v in c["n0"]))] + [
        Layout(H.shape[l], c["boxes"][l]) for l in range(1, nlev)]
    umac = [[lays[l].to_fabs(c["umac"][l][d], ng=1, face_dir=d, periodic=per) for d in range(dm)]
            for l in range(nlev)]
    phi = [lays[l].to_fabs(np.zeros(H.shape[l]), ng=1, periodic=per) for l in range(nlev)]
    rho = [lays[l].to_fabs(c["rho"][l], ng=2, periodic=per) for l in range(nlev)]
    rhs = [lays[l].to_fabs(c["macrhs"][l], ng=0, periodic=per) for l in range(nlev)]
    P = MacProjector(lays[0], c["dx0"], BcTower(c["bc_lo"], c["bc_hi"]), precision="fp64",
                     rel_eps=1e-13)
    try:
        P.set_amr(c["boxes"])
        st = P.macproject_ml(umac, phi, rho, macrhs=rhs, beta0=c["beta0"],
                             beta0_edge=c["beta0_edge"], ng_u=1, ng_phi=1, ng_rho=2, ng_rhs=0,
                             strict=True)
    finally:
        P.close()
    assert st["status"] == 0
    # compare the boxes' own faces and cells with the golden solution (phi up to the constant)
    ref_phi = [lays[l].to_fabs(c["phi"][l], ng=1, periodic=per) for l in range(nlev)]
    shift = None
    scale = max(np.max(np.abs(p)) for p in c["phi"])
    for l in range(nlev):
        for b, (lo, hi) in enumerate(lays[l].boxes):
            sl = tuple(slice(1, 1 + hi[d] - lo[d] + 1) for d in range(dm))
            diff = phi[l][b][sl] - ref_phi[l][b][sl]
            shift = diff.flat[0] if shift is None else shift
            assert np.max(np.abs(diff - shift)) <= 1e-9 * scale
            for d in range(dm):
                ref_u = lays[l].to_fabs(c["unew"][l][d], ng=1, face_dir=d, periodic=per)[b]
                slu = tuple(slice(1, 1 + hi[e] - lo[e] + 1 + (1 if e == d else 0)) for e in range(dm))
                den = np.max(np.abs(c["unew"][l][d][G.face_member(H, l, d)]))
                assert np.max(np.abs(umac[l][d][b][slu] - ref_u[slu])) <= 1e-9 * den
                if l == 0:
                    continue
                # create_umac_grown: the fine fabs' ghost faces inside the domain
                exp = O.create_umac_grown_fab(c["unew"][l][d], c["unew"][l - 1][d], H.inm[l], d,
                                              lo, hi, 1, per)
                m = ~np.isnan(exp)
                assert m.any()
                assert np.max(np.abs(umac[l][d][b][m] - exp[m])) <= 1e-9 * den
