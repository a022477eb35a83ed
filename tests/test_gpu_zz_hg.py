"""Nodal (HG) projection on the GPU (mac_hgproject_dense) against the golden direct solves and the
oracle: dense and cross stencils, 2-D and 3-D, periodic / wall / outflow faces, the initial,
pressure-iteration and regular projections with beta0, a nodal source and the alt energy fix.
The kernels' node arithmetic is the code tests/test_hg_host_exec.py runs on the host."""
import numpy as np
import pytest

import oracle as O
from maestro_gb300 import capi
from maestro_gb300.inputs import BC_DIR, BC_NEU, BC_PER
from maestro_gb300.macproject import BcTower, Layout, MacError, MacProjector
from tests.test_oracle_hg import G, _unknown_mask, load_hg

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _run(shape, dx, bc_lo, bc_hi, proj, dt, unew, uold, gpi, rhohalf, pi, b0=None, nodalrhs=None,
         dense=True, alt=False, rel_eps=1e-13, precision="fp64"):
    dev = torch.device("cuda", 0)
    t = lambda a: None if a is None else torch.from_numpy(  # noqa: E731
        np.ascontiguousarray(np.asarray(a, dtype=np.float64).transpose())).to(dev)
    tensors = [t(a) for a in (unew, uold, gpi, rhohalf, pi, b0, nodalrhs)]
    ptr = lambda x: 0 if x is None else x.data_ptr()  # noqa: E731
    dm = len(shape)
    P = MacProjector(Layout(shape, [((0,) * dm, tuple(v - 1 for v in shape))]), dx,
                     BcTower(bc_lo, bc_hi), precision=precision,
                     stream=torch.cuda.current_stream().cuda_stream, use_alt_energy_fix=int(alt))
    try:
        st = P.hgproject_dense(proj, dt, *[ptr(x) for x in tensors[:5]],
                               beta0_cart=ptr(tensors[5]) or None,
                               nodalrhs=ptr(tensors[6]) or None, dense_stencil=dense,
                               rel_eps=rel_eps, strict=True)
    finally:
        P.close()
    torch.cuda.synchronize()
    back = lambda x: np.asfortranarray(x.cpu().numpy().transpose())  # noqa: E731
    return back(tensors[0]), back(tensors[2]), back(tensors[4]), st


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", sorted(G.HG_CASES))
def test_hgproject_matches_golden(name, precision):
    c = load_hg(name)
    shape = c["rhohalf"].shape
    u, gpi, pi, st = _run(shape, c["dx"], c["bc_lo"], c["bc_hi"], int(c["proj"]), float(c["dt"]),
                          c["unew"], c["uold"], c["gpi"], c["rhohalf"], c["pi"],
                          b0=c.get("beta0"), nodalrhs=c.get("nodalrhs"), dense=bool(c["dense"]),
                          alt=bool(c["alt"]), precision=precision)
    assert st["status"] == 0 and st["rel_resid"] <= 1e-13
    assert np.max(np.abs(u - c["u_out"])) <= 1e-9 * np.max(np.abs(c["u_out"]))
    assert np.max(np.abs(gpi - c["gpi_out"])) <= 1e-9 * max(np.max(np.abs(c["gpi_out"])),
                                                             np.max(np.abs(c["gpi"])))
    m = _unknown_mask(shape, c["dx"], c["bc_lo"], c["bc_hi"])
    assert np.ptp((pi - c["pi_out"])[m]) <= 1e-9 * max(np.max(np.abs(c["pi_out"])), 1.0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("dense", [True, False])
def test_hgproject_matches_oracle_3d(dense, precision):
    rng = np.random.default_rng(23)
    shape = (32, 32, 32)
    dx = (1 / 32,) * 3
    bc = (BC_PER, BC_PER, BC_NEU)
    unew = rng.standard_normal(shape + (3,))
    gpi = rng.standard_normal(shape + (3,))
    rho = np.exp(0.3 * rng.standard_normal(shape))
    pi = np.zeros((33, 33, 33))
    u, g, p, st = _run(shape, dx, bc, bc, O.HG_REGULAR, 0.01, unew, unew, gpi, rho, pi,
                       dense=dense, rel_eps=O.EPS_HG, precision=precision)
    assert st["status"] == 0 and st["rel_resid"] <= O.EPS_HG
    uo, go, po, pho, so = O.hgproject(unew, unew, gpi, rho, pi, dx, bc, bc,
                                      proj_type=O.HG_REGULAR, dt=0.01, dense=dense,
                                      rel_eps=O.EPS_HG)
    assert np.max(np.abs(u - uo)) <= 1e-9 * np.max(np.abs(uo))
    assert np.max(np.abs(g - go)) <= 1e-9 * np.max(np.abs(go))


def test_hgproject_rejects_bad_input():
    shape = (8, 8)
    dx = (1 / 8, 1 / 8)
    bc = (BC_PER, BC_NEU)
    z = np.zeros(shape + (2,))
    rho = np.ones(shape)
    rho[3, 3] = 0.0
    with pytest.raises(MacError) as e:
        _run(shape, dx, bc, bc, O.HG_INITIAL, 1.0, z, z, z, rho, np.zeros((9, 9)))
    assert e.value.code == capi.MAC_ERR_BAD_DENSITY


@pytest.mark.parametrize("name", ["hg2d_32", "hg3d_12"])
def test_hgproject_on_host_fabs(name):
    # the drop-in form: per-box host fabs (several boxes, ghost cells / nodes) of every field
    from tests.test_hg_host_exec import make_fabs
    c = load_hg(name)
    shape = c["rhohalf"].shape
    dm = len(shape)
    per = [b == BC_PER for b in c["bc_lo"]]
    half = tuple(v // 2 for v in shape)
    lay = Layout.tiled(shape, half)
    boxes = lay.boxes
    fab = lambda a, nodal, ncomp=1: make_fabs(a, boxes, 1, nodal, per, ncomp)  # noqa: E731
    unew, uold, gpi = fab(c["unew"], 0, dm), fab(c["uold"], 0, dm), fab(c["gpi"], 0, dm)
    rho, b0 = fab(c["rhohalf"], 0), fab(c["beta0"], 0)
    pi, nr = fab(c["pi"], 1), fab(c["nodalrhs"], 1)
    P = MacProjector(lay, c["dx"], BcTower(c["bc_lo"], c["bc_hi"]), precision="fp64",
                     use_alt_energy_fix=int(c["alt"]))
    try:
        st = P.hgproject(int(c["proj"]), float(c["dt"]), unew, uold, gpi, rho, pi, beta0_cart=b0,
                         nodalrhs=nr, dense_stencil=bool(c["dense"]), rel_eps=1e-13,
                         strict=True)
    finally:
        P.close()
    assert st["status"] == 0
    ref_u, ref_g = fab(c["u_out"], 0, dm), fab(c["gpi_out"], 0, dm)
    ref_pi = fab(c["pi_out"], 1)
    su = np.max(np.abs(c["u_out"]))
    sg = max(np.max(np.abs(c["gpi_out"])), np.max(np.abs(c["gpi"])))
    shift = None
    for b, (lo, hi) in enumerate(boxes):
        sl = tuple(slice(1, 1 + hi[d] - lo[d] + 1) for d in range(dm))
        sn = tuple(slice(1, 1 + hi[d] - lo[d] + 2) for d in range(dm))
        assert np.max(np.abs(unew[b][sl] - ref_u[b][sl])) <= 1e-9 * su
        assert np.max(np.abs(gpi[b][sl] - ref_g[b][sl])) <= 1e-9 * sg
        dpi = pi[b][sn] - ref_pi[b][sn]
        shift = dpi.flat[0] if shift is None else shift
        assert np.max(np.abs(dpi - shift)) <= 1e-9 * max(np.max(np.abs(c["pi_out"])), 1.0)


def _pad_fabs(pad, boxes, ncomp=1):
    """Per-box fabs with one ghost layer cut from a whole-domain array that has one."""
    out = []
    for lo, hi in boxes:
        sl = tuple(slice(lo[d], hi[d] + 3) for d in range(len(lo)))
        out.append(np.asfortranarray(pad[sl], dtype=np.float64))
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", sorted(G.HG_INFLOW_CASES))
def test_hgproject_inflow_dense_matches_golden(name, precision):
    # inlet faces through mac_hgproject_dense_inflow (wall values on the device)
    from tests.test_oracle_hg import check_against_golden, load_inflow
    c = load_inflow(name)
    shape = c["rhohalf"].shape
    dm = len(shape)
    dev = torch.device("cuda", 0)
    t = lambda a: None if a is None else torch.from_numpy(  # noqa: E731
        np.ascontiguousarray(np.asarray(a, dtype=np.float64).transpose())).to(dev)
    tens = [t(c.get(k)) for k in ("unew", "uold", "gpi", "rhohalf", "pi", "beta0", "nodalrhs")]
    wall = torch.from_numpy(np.ascontiguousarray(c["wall"])).to(dev)
    ptr = lambda x: 0 if x is None else x.data_ptr()  # noqa: E731
    P = MacProjector(Layout(shape, [((0,) * dm, tuple(v - 1 for v in shape))]), c["dx"],
                     BcTower(c["bc_lo"], c["bc_hi"]), precision=precision,
                     stream=torch.cuda.current_stream().cuda_stream,
                     use_alt_energy_fix=int(c["alt"]))
    try:
        P.set_inflow(c["lo"], c["hi"])
        # an inlet needs its wall values
        with pytest.raises(MacError) as e:
            P.hgproject_dense(int(c["proj"]), float(c["dt"]), *[ptr(x) for x in tens[:5]],
                              strict=True)
        assert e.value.code == capi.MAC_ERR_INVALID
        st = P.hgproject_dense(int(c["proj"]), float(c["dt"]), *[ptr(x) for x in tens[:5]],
                               beta0_cart=ptr(tens[5]) or None, nodalrhs=ptr(tens[6]) or None,
                               dense_stencil=bool(c["dense"]), rel_eps=1e-13, strict=True,
                               inflow_wall=wall.data_ptr())
    finally:
        P.close()
    torch.cuda.synchronize()
    back = lambda x: np.asfortranarray(x.cpu().numpy().transpose())  # noqa: E731
    assert st["status"] == 0 and st["rel_resid"] <= 1e-13
    check_against_golden(c, back(tens[0]), back(tens[2]), back(tens[4]), None)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", sorted(G.HG_INFLOW_CASES))
def test_hgproject_inflow_on_host_fabs(name, precision):
    # the drop-in form: the inflow velocity in the ghost cells of the caller's fabs (four boxes)
    from tests.test_hg_host_exec import make_fabs
    from tests.test_oracle_hg import check_against_golden, load_inflow
    c = load_inflow(name)
    shape = c["rhohalf"].shape
    dm = len(shape)
    per = [b == BC_PER for b in c["bc_lo"]]
    lay = Layout.tiled(shape, tuple(v // 2 for v in shape))
    boxes = lay.boxes
    fab = lambda a, nodal, ncomp=1, ng=1: make_fabs(a, boxes, ng, nodal, per, ncomp)  # noqa: E731
    unew = _pad_fabs(c["unew_pad"], boxes)
    uold = _pad_fabs(c["uold_pad"], boxes)
    gpi, rho = fab(c["gpi"], 0, dm), fab(c["rhohalf"], 0)
    if "beta0_pad" in c:
        b0, ng_b0 = _pad_fabs(c["beta0_pad"], boxes), 1
    else:
        b0, ng_b0 = fab(c["beta0"], 0, ng=0), 0
    pi, nr = fab(c["pi"], 1), fab(c["nodalrhs"], 1)
    P = MacProjector(lay, c["dx"], BcTower(c["bc_lo"], c["bc_hi"]), precision=precision,
                     use_alt_energy_fix=int(c["alt"]))
    try:
        P.set_inflow(c["lo"], c["hi"])
        st = P.hgproject(int(c["proj"]), float(c["dt"]), unew, uold, gpi, rho, pi, beta0_cart=b0,
                         nodalrhs=nr, ng_b0=ng_b0, dense_stencil=bool(c["dense"]),
                         rel_eps=1e-13, strict=True)
    finally:
        P.close()
    assert st["status"] == 0
    ref_u, ref_g, ref_pi = fab(c["u_out"], 0, dm), fab(c["gpi_out"], 0, dm), fab(c["pi_out"], 1)
    su = np.max(np.abs(c["u_out"]))
    sg = max(np.max(np.abs(c["gpi_out"])), np.max(np.abs(c["gpi"])))
    shift = None
    for b, (lo, hi) in enumerate(boxes):
        sl = tuple(slice(1, 1 + hi[d] - lo[d] + 1) for d in range(dm))
        sn = tuple(slice(1, 1 + hi[d] - lo[d] + 2) for d in range(dm))
        assert np.max(np.abs(unew[b][sl] - ref_u[b][sl])) <= 1e-9 * su
        assert np.max(np.abs(gpi[b][sl] - ref_g[b][sl])) <= 1e-9 * sg
        dpi = pi[b][sn] - ref_pi[b][sn]
        shift = dpi.flat[0] if shift is None else shift
        assert np.max(np.abs(dpi - shift)) <= 1e-9 * max(np.max(np.abs(c["pi_out"])), 1.0)


def test_inflow_arguments_are_checked():
    shape = (8, 8)
    dx = (1 / 8, 1 / 8)
    lay = Layout(shape, [((0, 0), (7, 7))])
    P = MacProjector(lay, dx, BcTower((BC_PER, BC_NEU), (BC_PER, BC_DIR)), precision="fp64")
    try:
        for lo, hi in (((1, 0), (0, 0)), ((0, 0), (0, 1)), ((0, 2), (0, 0))):
            with pytest.raises(MacError) as e:   # periodic face, outflow face, bad flag
                P.set_inflow(lo, hi)
            assert e.value.code == capi.MAC_ERR_INVALID
        P.set_inflow((0, 1), (0, 0))
        z = [np.zeros((8, 8, 2), order="F")]
        with pytest.raises(MacError) as e:   # fabs without the ghost layer the inlet needs
            P.hgproject(O.HG_INITIAL, 1.0, z, None, z, [np.ones((8, 8), order="F")],
                        [np.zeros((9, 9), order="F")], ng_u=0, ng_gp=0, ng_rho=0, ng_pi=0,
                        strict=True)
        assert e.value.code == capi.MAC_ERR_INVALID
    finally:
        P.close()
