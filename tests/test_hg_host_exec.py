"""The library's nodal (HG) projection code executed on the host (no GPU).

tests/csrc/hg_host.cpp runs the node / cell functions and the hg::project sequencing of
maestro_gb300/csrc/hg_nodal.cuh -- what the CUDA kernels of hg_nodal.cu launch -- with loops, so
the nodal arithmetic and the V-cycle are checked against the golden direct solves and the oracle
before a GPU runs them."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from maestro_gb300.inputs import BC_DIR, BC_NEU, BC_PER
from tests.test_oracle_hg import G, _unknown_mask, load_hg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _opt_flags():
    """-O2; with MAESTRO_HOST_ASAN=1 an AddressSanitizer build instead (run pytest with
    LD_PRELOAD=$(gcc -print-file-name=libasan.so) ASAN_OPTIONS=detect_leaks=0): every array access
    of the library's cell functions is then bounds-checked on the host."""
    if os.environ.get("MAESTRO_HOST_ASAN") == "1":
        return ["-O1", "-g", "-fsanitize=address", "-fno-omit-frame-pointer"]
    return ["-O2"]


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("hgh") / "libhg_host.so")
    subprocess.run([cxx, *_opt_flags(), "-std=c++17", "-fPIC", "-shared", "-I",
                    os.path.join(ROOT, "maestro_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "csrc", "hg_host.cpp"), "-o", out],
                   check=True, capture_output=True)
    L = ctypes.CDLL(out)
    d = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    ci, cd = ctypes.c_int, ctypes.c_double
    L.hgh_project.argtypes = [ci, ip, d, ip, ip, ip, ci, ci, cd, ci, cd, ci, ci, ci, d, d, d, d,
                              d, d, d, d, d]
    L.hgh_project.restype = ci
    L.hgh_project_prec.argtypes = [ci, ip, d, ip, ip, ip, ci, ci, cd, ci, cd, ci, ci, ci, ci, d,
                                   d, d, d, d, d, d, d, d]
    L.hgh_project_prec.restype = ci
    L.hgh_fabs.argtypes = [ci, ip, ip, ci, ip, ci, ci, ci, ci, ctypes.POINTER(d), d]
    L.hgh_fabs.restype = None
    L.hgh_set_wall.argtypes = [ctypes.POINTER(ctypes.c_long), d]
    L.hgh_set_wall.restype = None
    return L


def run_host(L, shape, dx, bc_lo, bc_hi, proj, dt, unew, uold, gpi, rhohalf, pi, b0=None,
             nodalrhs=None, dense=True, alt=False, rel_eps=1e-13, max_cycles=200, inner=0):
    dm = len(shape)
    arr = lambda a: None if a is None else np.asfortranarray(a, dtype=np.float64)  # noqa: E731
    ptr = lambda a: None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    ia = lambda v: (ctypes.c_int * 3)(*(list(v) + [0] * (3 - len(v))))  # noqa: E731
    u = arr(unew).copy(order="F")
    g = arr(gpi).copy(order="F")
    p = arr(pi).copy(order="F")
    uo, rh, bb, nr = arr(uold), arr(rhohalf), arr(b0), arr(nodalrhs)
    phi = np.zeros(tuple(v + 1 for v in shape), order="F")
    st = (ctypes.c_double * 4)()
    rc = L.hgh_project_prec(dm, ia(shape), (ctypes.c_double * 3)(*(list(dx) + [1.0] * (3 - dm))),
                            ia([b == BC_PER for b in bc_lo]), ia([b == BC_DIR for b in bc_lo]),
                            ia([b == BC_DIR for b in bc_hi]), int(dense), int(proj), float(dt),
                            int(alt), rel_eps, max_cycles, 2, 2, int(inner), ptr(u), ptr(uo),
                            ptr(g), ptr(rh), ptr(p), ptr(bb), ptr(nr), ptr(phi), st)
    return rc, u, g, p, phi, list(st)


@pytest.mark.parametrize("inner", [0, 2])
@pytest.mark.parametrize("name", sorted(G.HG_CASES))
def test_library_hg_code_on_host_matches_golden(host_lib, name, inner):
    # inner = 0: the FP64 solve; inner = 2: FP32 V-cycles under FP64 refinement (mixed)
    c = load_hg(name)
    shape = c["rhohalf"].shape
    rc, u, gpi, pi, phi, st = run_host(host_lib, shape, c["dx"], c["bc_lo"], c["bc_hi"],
                                       int(c["proj"]), float(c["dt"]), c["unew"], c["uold"],
                                       c["gpi"], c["rhohalf"], c["pi"], b0=c.get("beta0"),
                                       nodalrhs=c.get("nodalrhs"), dense=bool(c["dense"]),
                                       alt=bool(c["alt"]), inner=inner)
    assert rc == 0 and st[2] <= 1e-13, st
    m = _unknown_mask(shape, c["dx"], c["bc_lo"], c["bc_hi"])
    a, b = phi[m], c["phi_out"][m]
    if BC_DIR not in c["bc_lo"] + c["bc_hi"]:
        a, b = a - a.mean(), b - b.mean()
    assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(b))
    assert np.max(np.abs(u - c["u_out"])) <= 1e-9 * np.max(np.abs(c["u_out"]))
    assert np.max(np.abs(gpi - c["gpi_out"])) <= 1e-9 * max(np.max(np.abs(c["gpi_out"])),
                                                             np.max(np.abs(c["gpi"])))
    # pi: the golden one up to the constant phi is fixed to (singular problems)
    dpi = (pi - c["pi_out"])[m]
    assert np.ptp(dpi) <= 1e-9 * max(np.max(np.abs(c["pi_out"])), 1.0)


@pytest.mark.parametrize("dense", [True, False])
@pytest.mark.parametrize("shape,bc", [((32, 32), (BC_PER, BC_NEU)), ((16, 16, 16), (BC_PER, BC_PER, BC_NEU)),
                                      ((24, 16), (BC_NEU, BC_DIR))])
def test_library_hg_code_on_host_matches_oracle_at_eps_hg(host_lib, dense, shape, bc):
    rng = np.random.default_rng(17)
    dm = len(shape)
    dx = tuple(1.0 / shape[0] for _ in shape)
    bc_lo, bc_hi = bc, bc
    unew = rng.standard_normal(shape + (dm,))
    gpi = np.zeros(shape + (dm,))
    rho = np.exp(0.3 * rng.standard_normal(shape))
    pi = np.zeros(tuple(v + 1 for v in shape))
    rc, u, g, p, phi, st = run_host(host_lib, shape, dx, bc_lo, bc_hi, O.HG_INITIAL, 1.0, unew,
                                    unew, gpi, rho, pi, dense=dense, rel_eps=O.EPS_HG)
    assert rc == 0 and st[2] <= O.EPS_HG
    uo, go, po, pho, so = O.hgproject(unew, unew, gpi, rho, pi, dx, bc_lo, bc_hi,
                                      proj_type=O.HG_INITIAL, dense=dense, rel_eps=O.EPS_HG)
    # both at eps_hg = 1e-12 on the same system (different bottom solvers): within 1e-9
    assert np.max(np.abs(u - uo)) <= 1e-9 * np.max(np.abs(uo))


def make_fabs(arr, boxes, ng, nodal, per, ncomp=1):
    """Per-box fabs (Fortran order, components last) cut from a whole-domain cell / node array;
    ghosts wrapped where periodic, clamped elsewhere."""
    dm = len(boxes[0][0])
    full = np.asarray(arr)
    ext = full.shape[:dm]
    out = []
    for lo, hi in boxes:
        idx = []
        for d in range(dm):
            r = np.arange(lo[d] - ng, hi[d] + 1 + nodal + ng)
            n = ext[d] - nodal
            r = np.where(r < 0, r + n, r) if per[d] else np.clip(r, 0, ext[d] - 1)
            r = np.where(r >= ext[d], r - n, r) if per[d] else r
            idx.append(r)
        sub = full[np.ix_(*idx)] if ncomp == 1 else full[np.ix_(*idx, np.arange(ncomp))]
        out.append(np.asfortranarray(sub))
    return out


@pytest.mark.parametrize("nodal,ncomp", [(0, 2), (1, 1)])
def test_hg_fab_mapping(host_lib, nodal, ncomp):
    shape = (16, 12)
    per = [True, False]
    boxes = [((0, 0), (7, 5)), ((8, 0), (15, 5)), ((0, 6), (7, 11)), ((8, 6), (15, 11))]
    rng = np.random.default_rng(2)
    ashape = tuple(v + nodal for v in shape) + ((ncomp,) if ncomp > 1 else ())
    arr = np.asfortranarray(rng.standard_normal(ashape))
    fabs = make_fabs(arr, boxes, 2, nodal, per, ncomp)
    flat = np.array([list(lo) + [0] + list(hi) + [0] for lo, hi in boxes], dtype=np.int32).ravel()
    ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))  # noqa: E731
    n = np.array(list(shape) + [1], dtype=np.int32)
    pe = np.array([1, 0, 0], dtype=np.int32)
    got = np.zeros_like(arr, order="F")
    host_lib.hgh_fabs(2, ip(n), ip(pe), len(boxes), ip(flat), 2, nodal, ncomp, 0,
                      O._ptr_array(fabs), got.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    # every cell / node of the domain belongs to some box (the last node row of a periodic
    # direction is the image and is written too)
    np.testing.assert_array_equal(got, arr)
    back = [np.zeros_like(f, order="F") for f in fabs]
    host_lib.hgh_fabs(2, ip(n), ip(pe), len(boxes), ip(flat), 2, nodal, ncomp, 1,
                      O._ptr_array(back), arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    for f, g, (lo, hi) in zip(back, fabs, boxes):
        sl = tuple(slice(2, 2 + hi[d] - lo[d] + 1 + nodal) for d in range(2))
        np.testing.assert_array_equal(f[sl], g[sl])
        mask = np.ones(f.shape, dtype=bool)
        mask[sl] = False
        assert np.all(f[mask] == 0.0)


def test_library_hg_code_reports_a_nonfinite_input(host_lib):
    shape = (16, 16)
    dx = (1 / 16, 1 / 16)
    bc = (BC_PER, BC_NEU)
    u = np.zeros(shape + (2,))
    u[5, 5, 0] = np.nan
    rc, *_ = run_host(host_lib, shape, dx, bc, bc, O.HG_INITIAL, 1.0, u, u, np.zeros_like(u),
                      np.ones(shape), np.zeros((17, 17)))
    assert rc < 0


@pytest.mark.parametrize("dense", [1, 0])
@pytest.mark.parametrize("dm,n,per,dlo,dhi", [
    (3, (6, 4, 8), (1, 1, 0), (0, 0, 0), (0, 0, 1)),
    (3, (2, 2, 2), (1, 1, 0), (0, 0, 0), (0, 0, 0)),
    (2, (8, 6), (1, 0), (0, 1), (0, 0)),
    (3, (1, 4, 4), (1, 0, 0), (0, 0, 1), (0, 0, 0)),
])
def test_node_row_reproduces_node_op(host_lib, dm, n, per, dlo, dhi, dense):
    """The row form of the nodal operator (used to build the dense inverse of the coarsest
    level) gives the same (L phi)_p as node_op on every node, periodic folds and Dirichlet faces
    included, to rounding."""
    L = host_lib
    L.hgh_row_check.restype = ctypes.c_double
    ia = lambda v: (ctypes.c_int * 3)(*(list(v) + [0] * (3 - len(v))))  # noqa: E731
    dx = (ctypes.c_double * 3)(*([0.5, 0.25, 0.125][:dm] + [1.0] * (3 - dm)))
    err = L.hgh_row_check(dm, ia(n), dx, ia(per), ia(dlo), ia(dhi), dense, 7)
    assert err <= 1e-14, err


@pytest.mark.parametrize("n", [2, 7, 16, 100, 128, 256, 384, 512, 1000, 4096])
def test_isotropic_dense_weights_of_the_axis_neighbours_are_exactly_zero(host_lib, n):
    """The GPU's dense 3-D kernels leave out the six axis neighbours on a level whose weights
    kw[1], kw[2], kw[4] are exactly 0 (fma(0, a, acc) = acc: bitwise the full stencil).  On an
    isotropic level they are, in FP64 and in the FP32 levels' rounding, for spacings that are
    not powers of two as well; on an anisotropic level they are not, and the kernels keep them."""
    L = host_lib
    kw64 = (ctypes.c_double * 8)()
    kw32 = (ctypes.c_float * 8)()
    for h in (1.0 / n, 0.7 / n, 3.0 / n):
        L.hgh_dense_weights(3, (ctypes.c_double * 3)(h, h, h), kw64, kw32)
        assert [kw64[m] for m in (1, 2, 4)] == [0.0, 0.0, 0.0]
        assert [kw32[m] for m in (1, 2, 4)] == [0.0, 0.0, 0.0]
        assert all(kw64[m] != 0.0 for m in (0, 3, 5, 6, 7))
    L.hgh_dense_weights(3, (ctypes.c_double * 3)(1.0 / n, 1.0 / n, 2.0 / n), kw64, kw32)
    assert any(kw64[m] != 0.0 for m in (1, 2, 4))


@pytest.mark.parametrize("inner", [0, 2])
@pytest.mark.parametrize("name", sorted(G.HG_INFLOW_CASES))
def test_library_hg_code_on_host_inflow_matches_golden(host_lib, name, inner):
    # inlet faces: the library's divergence with the wall values of the ghost cells
    from tests.test_oracle_hg import check_against_golden, load_inflow
    c = load_inflow(name)
    shape = c["rhohalf"].shape
    off, _ = O.hg_wall_layout(shape, c["lo"], c["hi"])
    wall = np.ascontiguousarray(c["wall"])
    host_lib.hgh_set_wall((ctypes.c_long * 6)(*off),
                          wall.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    try:
        rc, u, gpi, pi, phi, st = run_host(host_lib, shape, c["dx"], c["bc_lo"], c["bc_hi"],
                                           int(c["proj"]), float(c["dt"]), c["unew"], c["uold"],
                                           c["gpi"], c["rhohalf"], c["pi"], b0=c.get("beta0"),
                                           nodalrhs=c.get("nodalrhs"), dense=bool(c["dense"]),
                                           alt=bool(c["alt"]), inner=inner)
    finally:
        host_lib.hgh_set_wall(None, None)
    assert rc == 0 and st[2] <= 1e-13, st
    check_against_golden(c, u, gpi, pi, phi)
