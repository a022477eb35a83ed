"""ctypes binding of the C ABI in include/maestro_mac.h (libmaestro_mac.so).

This is plumbing only: every numerical operation runs in the CUDA library.  Loading fails loudly
when the library has not been built -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmaestro_mac.so")

MAC_OK = 0
MAC_ERR_INVALID = -1
MAC_ERR_CUDA = -2
MAC_ERR_NOT_CONVERGED = -3
MAC_ERR_NONFINITE = -4
MAC_ERR_ALLOC = -5
MAC_ERR_UNSUPPORTED = -6
MAC_ERR_BAD_DENSITY = -7
MAC_ERR_TOO_LARGE = -8
MAC_ERR_DEVICE_TIMEOUT = -9

MAC_BC_PER, MAC_BC_INT, MAC_BC_DIR, MAC_BC_NEU = -1, 0, 1, 2
MAC_PREC_FP64, MAC_PREC_MIXED = 0, 1
MAC_PTR_HOST, MAC_PTR_DEVICE = 0, 1
KT_NAMES = ("smooth", "restrict", "coarse", "prolong", "accum", "resid", "setup", "correct")

# Every symbol include/maestro_mac.h declares.
EXPORTED = (
    "mac_default_opts", "mac_strerror", "mac_version", "mac_ctx_create", "mac_ctx_destroy",
    "mac_ctx_set_opts", "mac_ctx_levels", "mac_macproject", "mac_multigrid",
    "mac_macproject_dense", "mac_macproject_adjoint_dense", "mac_cell_to_edge",
    "mac_solve_small_noalloc", "mac_make_macrhs", "mac_make_macrhs_dense", "mac_make_at_halftime",
    "mac_macproject_cart", "mac_macproject_cart_dense", "mac_ctx_set_amr",
    "mac_macproject_ml_dense", "mac_macproject_ml", "mac_hgproject_dense", "mac_hgproject",
    "mac_ctx_set_inflow", "mac_hgproject_dense_inflow",
)
MAC_NOALLOC_MAX_CELLS = 4096


class MacGeom(ctypes.Structure):
    _fields_ = [
        ("dm", ctypes.c_int),
        ("domain_lo", ctypes.c_int * 3),
        ("domain_hi", ctypes.c_int * 3),
        ("dx", ctypes.c_double * 3),
        ("bc_lo", ctypes.c_int * 3),
        ("bc_hi", ctypes.c_int * 3),
        ("nboxes", ctypes.c_int),
        ("box_lo", ctypes.POINTER(ctypes.c_int)),
        ("box_hi", ctypes.POINTER(ctypes.c_int)),
    ]


class MacOpts(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int),
        ("use_alt_energy_fix", ctypes.c_int),
        ("rel_eps", ctypes.c_double),
        ("abs_eps", ctypes.c_double),
        ("max_vcycles", ctypes.c_int),
        ("nu1", ctypes.c_int),
        ("nu2", ctypes.c_int),
        ("nub", ctypes.c_int),
        ("bottom_eps", ctypes.c_double),
        ("bottom_max_iter", ctypes.c_int),
        ("max_levels", ctypes.c_int),
        ("use_graph", ctypes.c_int),
        ("verbose", ctypes.c_int),
        ("timing", ctypes.c_int),
        ("inner_vcycles", ctypes.c_int),
        ("coarse_tail", ctypes.c_int),
        ("adaptive_inner", ctypes.c_int),
        ("inner_krylov", ctypes.c_int),
        ("inner_nu1", ctypes.c_int),
        ("inner_nu2", ctypes.c_int),
        ("inner_exact_bottom", ctypes.c_int),
        ("inner_omega", ctypes.c_double),
        ("wait_limit_s", ctypes.c_double),
        ("inject_wait_expiry", ctypes.c_int),
        ("fused_sweep", ctypes.c_int),
    ]


class MacStats(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int),
        ("vcycles", ctypes.c_int),
        ("refine_iters", ctypes.c_int),
        ("nlevels", ctypes.c_int),
        ("bottom_iters", ctypes.c_int),
        ("fnorm", ctypes.c_double),
        ("resid0", ctypes.c_double),
        ("rel_resid", ctypes.c_double),
        ("nhist", ctypes.c_int),
        ("hist", ctypes.c_double * 64),
        ("setup_ms", ctypes.c_double),
        ("solve_ms", ctypes.c_double),
        ("total_ms", ctypes.c_double),
        ("launches", ctypes.c_longlong),
        ("ktime_ms", ctypes.c_double * 8),
        ("ktime_launches", ctypes.c_int * 8),
    ]

    def as_dict(self):
        return {
            "status": self.status,
            "vcycles": self.vcycles,
            "refine_iters": self.refine_iters,
            "nlevels": self.nlevels,
            "bottom_iters": self.bottom_iters,
            "fnorm": self.fnorm,
            "resid0": self.resid0,
            "rel_resid": self.rel_resid,
            "hist": [self.hist[i] for i in range(self.nhist)],
            "setup_ms": self.setup_ms,
            "solve_ms": self.solve_ms,
            "total_ms": self.total_ms,
            "launches": self.launches,
            "ktime_ms": [self.ktime_ms[i] for i in range(8)],
            "ktime_launches": [self.ktime_launches[i] for i in range(8)],
        }


class MacError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        super().__init__(f"{where}: {code} ({strerror(code)})")


_lib = None


def lib_loaded() -> bool:
    return _lib is not None


def lib():
    """Load libmaestro_mac.so (raises if it was not built; build() in __graft_entry__)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"CUDA library not built: {LIB_PATH} (run maestro_gb300.build.build())")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    dp = P(ctypes.c_double)
    dpp = P(P(ctypes.c_double))
    L.mac_default_opts.argtypes = [P(MacOpts)]
    L.mac_default_opts.restype = None
    L.mac_strerror.argtypes = [ctypes.c_int]
    L.mac_strerror.restype = ctypes.c_char_p
    L.mac_version.argtypes = []
    L.mac_version.restype = ctypes.c_char_p
    L.mac_ctx_create.argtypes = [P(vp), P(MacGeom), P(MacOpts), vp]
    L.mac_ctx_create.restype = ctypes.c_int
    L.mac_ctx_destroy.argtypes = [vp]
    L.mac_ctx_destroy.restype = ctypes.c_int
    L.mac_ctx_set_opts.argtypes = [vp, P(MacOpts)]
    L.mac_ctx_set_opts.restype = ctypes.c_int
    L.mac_ctx_levels.argtypes = [vp, P(ctypes.c_int)]
    L.mac_ctx_levels.restype = ctypes.c_int
    L.mac_macproject.argtypes = [vp, ctypes.c_int, dpp, ctypes.c_int, dpp, ctypes.c_int, dpp,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_int, dpp, ctypes.c_int, dp,
                                 dp, P(MacStats)]
    L.mac_macproject.restype = ctypes.c_int
    L.mac_multigrid.argtypes = [vp, ctypes.c_int, dpp, ctypes.c_int, dpp, ctypes.c_int, dpp,
                                ctypes.c_int, dpp, ctypes.c_int, P(MacStats)]
    L.mac_multigrid.restype = ctypes.c_int
    L.mac_macproject_dense.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, P(MacStats)]
    L.mac_macproject_dense.restype = ctypes.c_int
    L.mac_macproject_cart.argtypes = [vp, ctypes.c_int, dpp, ctypes.c_int, dpp, ctypes.c_int,
                                      dpp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dpp,
                                      ctypes.c_int, dpp, ctypes.c_int, P(MacStats)]
    L.mac_macproject_cart.restype = ctypes.c_int
    L.mac_macproject_cart_dense.argtypes = [vp] * 10 + [P(MacStats)]
    L.mac_macproject_cart_dense.restype = ctypes.c_int
    L.mac_macproject_adjoint_dense.argtypes = [vp] + [vp] * 17 + [P(MacStats)]
    L.mac_macproject_adjoint_dense.restype = ctypes.c_int
    L.mac_cell_to_edge.argtypes = [ctypes.c_int, dp, dp]
    L.mac_cell_to_edge.restype = ctypes.c_int
    ip = P(ctypes.c_int)
    L.mac_solve_small_noalloc.argtypes = [ctypes.c_int, ip, dp, ip, ip, vp, vp, vp, vp, vp, vp,
                                          ctypes.c_double, ctypes.c_int, vp, P(MacStats)]
    L.mac_solve_small_noalloc.restype = ctypes.c_int
    ci, cd = ctypes.c_int, ctypes.c_double
    L.mac_make_macrhs.argtypes = [vp, ci, dpp, ci, dpp, ci, dpp, ci, dp, dp, dp, dp, dpp, ci, dpp,
                                  ci, cd, cd, ci, ci]
    L.mac_make_macrhs.restype = ci
    L.mac_make_macrhs_dense.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, cd, cd, ci, ci]
    L.mac_make_macrhs_dense.restype = ci
    L.mac_make_at_halftime.argtypes = [vp, ci, dpp, ci, ci, ci, dpp, ci, dpp, ci, ci, ci]
    L.mac_make_at_halftime.restype = ci
    vpp = P(vp)
    L.mac_ctx_set_amr.argtypes = [vp, ci, ip, ip, ip]
    L.mac_ctx_set_amr.restype = ci
    L.mac_macproject_ml_dense.argtypes = [vp, vpp, vpp, vpp, vpp, vpp, vpp, P(MacStats)]
    L.mac_macproject_ml_dense.restype = ci
    L.mac_macproject_ml.argtypes = list(L.mac_macproject.argtypes)
    L.mac_macproject_ml.restype = ci
    L.mac_hgproject_dense.argtypes = [vp, ci, cd, ci, cd, vp, vp, vp, vp, vp, vp, vp, P(MacStats)]
    L.mac_hgproject_dense.restype = ci
    L.mac_hgproject.argtypes = [vp, ci, ci, cd, ci, cd, dpp, ci, dpp, ci, dpp, ci, dpp, ci, dpp, ci,
                                dpp, ci, dpp, ci, P(MacStats)]
    L.mac_hgproject.restype = ci
    L.mac_ctx_set_inflow.argtypes = [vp, ip, ip]
    L.mac_ctx_set_inflow.restype = ci
    L.mac_hgproject_dense_inflow.argtypes = [vp, ci, cd, ci, cd, vp, vp, vp, vp, vp, vp, vp, vp,
                                             P(MacStats)]
    L.mac_hgproject_dense_inflow.restype = ci
    _lib = L
    return L


def strerror(code: int) -> str:
    try:
        return lib().mac_strerror(int(code)).decode()
    except Exception:  # library missing
        return "unknown"


def default_opts(**kw) -> MacOpts:
    o = MacOpts()
    lib().mac_default_opts(ctypes.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(k)
        setattr(o, k, v)
    return o
