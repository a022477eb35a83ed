"""The library's multi-level projection code executed on the host (no GPU).

tests/csrc/amr_host.cpp runs the per-cell functions and the amr_project / amr_solve sequencing of
maestro_gb300/csrc/mac_amr.cuh -- what the CUDA kernels of mac_amr.cu launch -- with loops over
the cells, so the composite arithmetic and the cycle order are checked against the golden direct
solves before any GPU runs them."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from maestro_gb300.inputs import AMR_CASES
from tests.test_oracle_amr import G, load_amr, phi_err, u_err

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
    out = str(tmp_path_factory.mktemp("amrh") / "libamr_host.so")
    cmd = [cxx, *_opt_flags(), "-std=c++17", "-fPIC", "-fopenmp", "-shared",
           "-I", os.path.join(ROOT, "maestro_gb300", "csrc"), "-I", os.path.join(ROOT, "oracle"),
           os.path.join(ROOT, "tests", "csrc", "amr_host.cpp"),
           os.path.join(ROOT, "oracle", "mac_oracle.cpp"), "-o", out]
    subprocess.run(cmd, check=True, capture_output=True)
    L = ctypes.CDLL(out)
    P = ctypes.POINTER
    pd = P(P(ctypes.c_double))
    ip = P(ctypes.c_int)
    L.amrh_macproject.argtypes = [P(O.OrcOpts), ctypes.c_int, ip, ip, pd, pd, pd, pd, pd, pd,
                                  P(ctypes.c_double)]
    L.amrh_macproject.restype = ctypes.c_int
    L.amrh_macproject_prec.argtypes = [P(O.OrcOpts), ctypes.c_int, ip, ip, pd, pd, pd, pd, pd, pd,
                                       ctypes.c_int, ctypes.c_int, P(ctypes.c_double)]
    L.amrh_macproject_prec.restype = ctypes.c_int
    L.amrh_fabs.argtypes = [P(O.OrcOpts), ctypes.c_int, ip, ip, ctypes.c_int, ctypes.c_int,
                            ctypes.c_int, ctypes.c_int, ctypes.c_int, pd, P(ctypes.c_double)]
    L.amrh_fabs.restype = None
    L.amrh_check_colour_map.argtypes = [ctypes.c_int, ip, ip]
    L.amrh_check_colour_map.restype = ctypes.c_int
    return L


def run_host(L, c, rel_eps, inner=0, fab_inputs=False):
    nlev = c["nlev"]
    dm = c["dm"]
    phi = [np.zeros_like(p, order="F") for p in c["phi"]]
    u = [[np.array(x, order="F") for x in c["umac"][l]] for l in range(nlev)]
    up = []
    for l in range(nlev):
        for d in range(3):
            up.append(u[l][d] if d < dm else None)
    rho = [np.asfortranarray(r) for r in c["rho"]]
    mr = [np.asfortranarray(m) for m in c["macrhs"]]
    b0 = [np.ascontiguousarray(b) for b in c["beta0"]]
    b0e = [np.ascontiguousarray(b) for b in c["beta0_edge"]]
    o = O._opts(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], O.nlevels_for_boxes([c["n0"]]),
                rel_eps, -1.0, 200, 2, 2, 10, O.EPS_MAC_BOTTOM, 200, False, 0)
    nb, bx = O._ml_layout(c["n0"], c["boxes"])
    st = (ctypes.c_double * 4)()
    rc = L.amrh_macproject_prec(ctypes.byref(o), nlev,
                                nb.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                bx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), O._ptr_array(up),
                                O._ptr_array(phi), O._ptr_array(rho), O._ptr_array(mr),
                                O._ptr_array(b0), O._ptr_array(b0e), int(inner), int(fab_inputs),
                                st)
    return rc, u, phi, list(st)


@pytest.mark.parametrize("inner", [0, 2])
@pytest.mark.parametrize("name", sorted(AMR_CASES))
def test_library_amr_code_on_host_matches_golden(host_lib, name, inner):
    # inner = 0: the FP64 solve; inner = 2: FP32 multi-level cycles under FP64 refinement
    c = load_amr(name)
    H = G.Hierarchy(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"])
    rc, u, phi, st = run_host(host_lib, c, 1e-12, inner=inner)
    assert rc == 0 and st[2] <= 1e-12, st
    assert phi_err(H, phi, c["phi"]) <= 1e-9
    assert u_err(H, u, c["unew"]) <= 1e-9


@pytest.mark.parametrize("inner", [0, 2])
@pytest.mark.parametrize("name", sorted(AMR_CASES))
def test_library_amr_code_reads_only_what_the_fab_entry_defines(host_lib, name, inner):
    # the per-box entry defines a fine level's faces and cells only inside its boxes (density:
    # one ghost cell deeper); the rest of its arrays, and every work array, is NaN here
    c = load_amr(name)
    H = G.Hierarchy(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"])
    rc, u, phi, st = run_host(host_lib, c, 1e-12, inner=inner, fab_inputs=True)
    assert rc == 0 and st[2] <= 1e-12, st
    assert phi_err(H, phi, c["phi"]) <= 1e-9
    assert u_err(H, u, c["unew"]) <= 1e-9


@pytest.mark.parametrize("name", ["amr2d_3lev", "amr3d_16"])
def test_library_amr_code_on_host_matches_oracle_at_maestro_tolerance(host_lib, name):
    c = load_amr(name)
    H = G.Hierarchy(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"])
    eps = O.ml_rel_eps(c["nlev"])
    rc, u, phi, st = run_host(host_lib, c, eps)
    assert rc == 0 and st[2] <= eps
    uo, po, so = O.macproject_ml(c["umac"], [np.zeros_like(p) for p in c["phi"]], c["rho"],
                                 c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"],
                                 macrhs=c["macrhs"], beta0=c["beta0"],
                                 beta0_edge=c["beta0_edge"], rel_eps=eps)
    # same algorithm, same cycle count; only the level-0 correction differs in rounding
    assert int(st[1]) == so["vcycles"]
    assert phi_err(H, phi, po) <= 1e-10
    assert u_err(H, u, uo) <= 1e-10


@pytest.mark.parametrize("dir_", [-1, 0, 1])
def test_fab_gather_and_scatter_of_a_fine_level(host_lib, dir_):
    # level 1 of the layout with a box wrapping the periodic x boundary and one on the wall
    from maestro_gb300.macproject import Layout
    c = load_amr("amr2d_wrap")
    H = G.Hierarchy(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], c["boxes"])
    shape = list(H.shape[1])
    if dir_ >= 0:
        shape[dir_] += 1
    rng = np.random.default_rng(3)
    arr = np.asfortranarray(rng.standard_normal(shape))
    ng = 2
    lay = Layout(H.shape[1], c["boxes"][1])
    per = [b == O.BC_PER for b in c["bc_lo"]]
    fabs = lay.to_fabs(arr, ng=ng, face_dir=None if dir_ < 0 else dir_, periodic=per)
    o = O._opts(c["n0"], c["dx0"], c["bc_lo"], c["bc_hi"], 1, 0, 0, 0, 0, 0, 0, 0, 0, False, 0)
    nb, bx = O._ml_layout(c["n0"], c["boxes"])
    ipp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))  # noqa: E731
    level = np.zeros(shape, order="F")
    host_lib.amrh_fabs(ctypes.byref(o), 2, ipp(nb), ipp(bx), 1, dir_, ng, 1, 0,
                       O._ptr_array(fabs), level.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if dir_ < 0:
        # the boxes' cells and their ng ghost layers (corners included) that lie in the domain,
        # periodic images wrapped -- as far as the level stores cells: the bounding box of its
        # boxes grown by one cell (the whole extent of a periodic direction it would cross)
        want = np.zeros(H.shape[1], dtype=bool)
        for lo, hi in c["boxes"][1]:
            idx = []
            for d in range(2):
                r = np.arange(lo[d] - ng, hi[d] + 1 + ng)
                r = r % H.shape[1][d] if per[d] else r[(r >= 0) & (r < H.shape[1][d])]
                idx.append(r)
            want[np.ix_(*idx)] = True
        stored = np.ones(H.shape[1], dtype=bool)
        for d in range(2):
            a = min(lo[d] for lo, _ in c["boxes"][1]) - 1
            b = max(hi[d] for _, hi in c["boxes"][1]) + 1
            n = H.shape[1][d]
            if per[d] and (a < 0 or b > n - 1):
                a, b = 0, n - 1
            a, b = max(a, 0), min(b, n - 1)
            sl = [slice(None)] * 2
            keep = np.zeros(n, dtype=bool)
            keep[a:b + 1] = True
            stored &= keep.reshape([-1 if e == d else 1 for e in range(2)])
        want &= stored
    else:
        want = G.face_member(H, 1, dir_)
    np.testing.assert_array_equal(level[want], arr[want])
    assert np.all(level[~want] == 0.0)
    # scatter: the boxes' own entries of every fab come from the level array
    out = [np.zeros_like(f) for f in fabs]
    host_lib.amrh_fabs(ctypes.byref(o), 2, ipp(nb), ipp(bx), 1, dir_, ng, 0, 1,
                       O._ptr_array(out), arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    for f, g, (lo, hi) in zip(out, fabs, c["boxes"][1]):
        sl = tuple(slice(ng, ng + hi[d] - lo[d] + 1 + (1 if d == dir_ else 0)) for d in range(2))
        np.testing.assert_array_equal(f[sl], g[sl])
        mask = np.ones(f.shape, dtype=bool)
        mask[sl] = False
        assert np.all(f[mask] == 0.0)


def test_library_amr_code_reports_a_nonfinite_input(host_lib):
    # a NaN velocity reaches the right-hand side: the driver stops with its non-finite status
    # (the C entry turns it into MAC_ERR_NONFINITE) instead of cycling on NaNs
    c = load_amr("amr2d_32")
    c["umac"] = [[np.array(x, order="F") for x in c["umac"][l]] for l in range(c["nlev"])]
    c["umac"][1][0][30, 20] = np.nan
    rc, u, phi, st = run_host(host_lib, c, 1e-10)
    assert rc < 0


@pytest.mark.parametrize("dm,lo,ext", [(2, (0, 0), (8, 8)), (2, (3, 5), (7, 9)), (2, (1, 0), (1, 5)),
                                       (3, (0, 0, 0), (6, 6, 6)), (3, (5, 2, 7), (9, 4, 11)),
                                       (3, (2, 3, 1), (1, 1, 3))])
def test_smoother_colour_map_covers_each_colour_once(host_lib, dm, lo, ext):
    # the compact GS-RB launch: one thread per cell of the colour, odd extents and offset boxes
    ia = lambda v: (ctypes.c_int * 3)(*(list(v) + [0] * (3 - len(v))))  # noqa: E731
    assert host_lib.amrh_check_colour_map(dm, ia(lo), ia(ext)) == 0


@pytest.mark.parametrize("lo,ext", [((0, 0, 0), (130, 130, 130)), ((5, 3, 7), (37, 11, 9)),
                                    ((63, 0, 1), (1, 70, 3)), ((0, 0, 0), (2, 1, 1)),
                                    ((11, 2, 0), (13, 17, 1))])
def test_index_coordinates_match_64_bit_arithmetic(host_lib, lo, ext):
    """The level helpers' 32-bit divisions (cell, face and colour coordinates) give the 64-bit
    arithmetic's results on every index of the array box, odd extents and 2-D boxes included."""
    L = host_lib
    L.amrh_coords_check.restype = ctypes.c_long
    ia = lambda v: (ctypes.c_int * 3)(*v)  # noqa: E731
    assert L.amrh_coords_check(ia(lo), ia(ext)) == 0

