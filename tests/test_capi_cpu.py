"""C-ABI library checks that need no GPU: it loads, exports every symbol the header declares,
rejects invalid arguments before touching the device, and its host-only routine matches the
oracle."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import oracle as O
from maestro_gb300 import capi
from maestro_gb300.build import build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "maestro_mac.h")


@pytest.fixture(scope="module")
def lib():
    build()
    return capi.lib()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mac_[a-z0-9_]+)\s*\(", src)))


def test_header_and_binding_agree():
    assert declared_functions() == sorted(capi.EXPORTED)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", capi.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    syms = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    for f in declared_functions():
        assert f in syms, f
        assert hasattr(lib, f)


def test_strerror_and_defaults(lib):
    for code in (0, -1, -2, -3, -4, -5, -6, -7, -8):
        assert len(capi.strerror(code)) > 0
    o = capi.default_opts()
    # MAESTRO's MAC settings: eps_mac, V(2,2), mg_bottom_nu, eps_mac_bottom
    assert o.rel_eps == 1e-10 and o.nu1 == 2 and o.nu2 == 2 and o.nub == 10
    assert o.bottom_eps == 1e-3 and o.precision == capi.MAC_PREC_FP64 and o.abs_eps < 0


def test_invalid_geometry_rejected_without_device(lib):
    ctx = ctypes.c_void_p()
    g = capi.MacGeom()
    g.dm = 4
    assert lib.mac_ctx_create(ctypes.byref(ctx), ctypes.byref(g), None, None) == capi.MAC_ERR_INVALID
    # boxes that do not tile the domain
    g.dm = 2
    g.domain_hi[0] = 7
    g.domain_hi[1] = 7
    g.dx[0] = g.dx[1] = 1.0 / 8
    g.bc_lo[0] = g.bc_hi[0] = capi.MAC_BC_PER
    g.bc_lo[1] = g.bc_hi[1] = capi.MAC_BC_NEU
    lo = (ctypes.c_int * 3)(0, 0, 0)
    hi = (ctypes.c_int * 3)(3, 7, 0)
    g.nboxes = 1
    g.box_lo = ctypes.cast(lo, ctypes.POINTER(ctypes.c_int))
    g.box_hi = ctypes.cast(hi, ctypes.POINTER(ctypes.c_int))
    assert lib.mac_ctx_create(ctypes.byref(ctx), ctypes.byref(g), None, None) == capi.MAC_ERR_INVALID
    # periodic on one side only
    hi[0] = 7
    g.bc_hi[0] = capi.MAC_BC_NEU
    assert lib.mac_ctx_create(ctypes.byref(ctx), ctypes.byref(g), None, None) == capi.MAC_ERR_INVALID
    assert lib.mac_ctx_destroy(None) == capi.MAC_ERR_INVALID
    assert lib.mac_macproject_dense(None, *([None] * 8), None) == capi.MAC_ERR_INVALID
    assert lib.mac_macproject_cart_dense(None, *([None] * 9), None) == capi.MAC_ERR_INVALID
    assert lib.mac_macproject_cart(None, capi.MAC_PTR_HOST, None, 1, None, 1, None, 1, 1, 0,
                                   None, 0, None, 1, None) == capi.MAC_ERR_INVALID
    assert lib.mac_ctx_set_amr(None, 2, None, None, None) == capi.MAC_ERR_INVALID
    assert lib.mac_hgproject_dense(None, 1, 1.0, 1, 0.0, *([None] * 7), None) == capi.MAC_ERR_INVALID
    assert lib.mac_hgproject(None, capi.MAC_PTR_HOST, 1, 1.0, 1, 0.0, None, 1, None, 1, None, 1,
                             None, 1, None, 1, None, 1, None, 1, None) == capi.MAC_ERR_INVALID
    assert lib.mac_macproject_ml_dense(None, None, None, None, None, None, None,
                                       None) == capi.MAC_ERR_INVALID


def test_invalid_inner_options_rejected_without_device(lib):
    # options are checked before anything touches a device
    ctx = ctypes.c_void_p()
    g = capi.MacGeom()
    g.dm = 2
    g.domain_hi[0] = 7
    g.domain_hi[1] = 7
    g.dx[0] = g.dx[1] = 1.0 / 8
    g.bc_lo[0] = g.bc_hi[0] = capi.MAC_BC_PER
    g.bc_lo[1] = g.bc_hi[1] = capi.MAC_BC_NEU
    lo = (ctypes.c_int * 3)(0, 0, 0)
    hi = (ctypes.c_int * 3)(7, 7, 0)
    g.nboxes = 1
    g.box_lo = ctypes.cast(lo, ctypes.POINTER(ctypes.c_int))
    g.box_hi = ctypes.cast(hi, ctypes.POINTER(ctypes.c_int))
    for bad in (dict(inner_omega=0.0), dict(inner_omega=2.0), dict(inner_omega=float("nan")),
                dict(inner_nu1=-2), dict(inner_nu2=-3), dict(nu1=-1)):
        o = capi.default_opts(precision=capi.MAC_PREC_MIXED, **bad)
        rc = lib.mac_ctx_create(ctypes.byref(ctx), ctypes.byref(g), ctypes.byref(o), None)
        assert rc == capi.MAC_ERR_INVALID, bad


def test_cell_to_edge_matches_oracle(lib):
    from maestro_gb300.macproject import cell_to_edge
    b = 1e7 ** (1 / 1.4) * np.exp(-np.linspace(0, 4, 64) / 1.4)
    np.testing.assert_array_equal(cell_to_edge(b), O.cell_to_edge(b))


def test_mixed_precision_inner_defaults(lib):
    o = capi.default_opts()
    # inner FP32 V(2,1)-cycles with over-relaxed half-sweeps, at most 3 a refinement step,
    # adaptive count, exact bottom; the flexible-CG combination is opt-in
    assert (o.inner_nu1, o.inner_nu2, o.inner_vcycles) == (2, 1, 3)
    assert o.inner_omega == 1.25 and o.adaptive_inner == 1 and o.inner_exact_bottom == 1
    assert o.inner_krylov == 0 and o.coarse_tail == 1


def test_ctypes_structs_match_the_c_header(tmp_path):
    # the ctypes mirrors (and so the Fortran bind(C) types written from the same header) must
    # have the C layout: sizes and every field offset, from the header compiled by the C compiler
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"mac_opts": capi.MacOpts, "mac_stats": capi.MacStats, "mac_geom": capi.MacGeom}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "maestro_mac.h"',
             "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln.strip():
            parts = ln.split()
            got[(parts[0], parts[1])] = int(parts[2])
    for cname, cls in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)
