"""ctypes binding of libcfgpu.so (the C ABI in include/cajitafluids_gb300.h).

The library is loaded from the package directory (an in-tree build).  There
is no fallback: if the shared library is missing the import of the binding
fails loudly, because the CUDA path is the product.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcfgpu.so")

CF_OK = 0
CF_ERR_INVALID = -1
CF_ERR_CUDA = -2
CF_ERR_UNSUPPORTED = -3
CF_ERR_NOT_CONVERGED = -4
CF_ERR_NUMERIC = -5
CF_ERR_NOMEM = -6
CF_ERR_MESH = -7
CF_ERR_TOO_LARGE = -8
CF_ERR_TIMEOUT = -9
CF_NOALLOC_MAX_UNITS = 65536
CF_STRIP_FIELDS = 18

ERROR_NAMES = {
    CF_ERR_INVALID: "CF_ERR_INVALID",
    CF_ERR_CUDA: "CF_ERR_CUDA",
    CF_ERR_UNSUPPORTED: "CF_ERR_UNSUPPORTED",
    CF_ERR_NOT_CONVERGED: "CF_ERR_NOT_CONVERGED",
    CF_ERR_NUMERIC: "CF_ERR_NUMERIC",
    CF_ERR_NOMEM: "CF_ERR_NOMEM",
    CF_ERR_MESH: "CF_ERR_MESH",
    CF_ERR_TOO_LARGE: "CF_ERR_TOO_LARGE",
    CF_ERR_TIMEOUT: "CF_ERR_TIMEOUT",
}

CF_FIELD_QUANTITY = 0
CF_FIELD_U = 1
CF_FIELD_V = 2
CF_FIELD_PRESSURE = 3

CF_BC_SOLID = 0
CF_BC_FREE = 1

CF_PREC_FP64 = 0
CF_PREC_MIXED = 1

CF_FIX_Q1 = 1
CF_FIX_Q3 = 2

CF_SOLVE_CONVERGED = 0
CF_SOLVE_MAX_ITER = 1
CF_SOLVE_BREAKDOWN = 2
CF_SOLVE_NAN = 3
CF_SOLVE_TIMEOUT = 4


class GridDesc(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("lo", ctypes.c_double * 2), ("hi", ctypes.c_double * 2),
        ("periodic", ctypes.c_int * 2),
        ("precision", ctypes.c_int), ("device", ctypes.c_int),
    ]


class SolverOpts(ctypes.Structure):
    _fields_ = [
        ("solver", ctypes.c_char_p), ("precon", ctypes.c_char_p),
        ("tol", ctypes.c_double), ("abs_tol", ctypes.c_double),
        ("max_iter", ctypes.c_int),
        ("inner_tol", ctypes.c_double), ("max_outer", ctypes.c_int),
    ]


class SolveStats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int), ("outer_iterations", ctypes.c_int),
        ("status", ctypes.c_int),
        ("b_norm", ctypes.c_double), ("r_norm", ctypes.c_double),
        ("div_l2", ctypes.c_double), ("div_linf", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Profile(ctypes.Structure):
    _fields_ = [
        ("solve_ms", ctypes.c_double), ("solve_iters", ctypes.c_longlong), ("solve_batches", ctypes.c_longlong),
        ("advect_ms", ctypes.c_double), ("advect_calls", ctypes.c_longlong),
        ("project_ms", ctypes.c_double), ("projects", ctypes.c_longlong),
        ("adj_advect_ms", ctypes.c_double), ("adj_advect_calls", ctypes.c_longlong),
        ("adj_projects", ctypes.c_longlong), ("adj_iters", ctypes.c_longlong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


CF_CG_BATCH = 32

# exported symbol -> (restype, argtypes); the list is the ABI surface
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_pd = ctypes.c_ssize_t
SIGNATURES = {
    "cf_abi_version": (ctypes.c_int, []),
    "cf_ctx_create": (ctypes.c_int, [ctypes.POINTER(GridDesc), ctypes.POINTER(_vp)]),
    "cf_ctx_destroy": (ctypes.c_int, [_vp]),
    "cf_last_error": (ctypes.c_char_p, [_vp]),
    "cf_owned_extent": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _ip]),
    "cf_cell_size": (ctypes.c_int, [_vp, _dp]),
    "cf_set_bc": (ctypes.c_int, [_vp, _ip]),
    "cf_set_source": (ctypes.c_int, [_vp, _dp, _dp, _dp, ctypes.c_double, ctypes.c_int]),
    "cf_set_body_force": (ctypes.c_int, [_vp, _dp, ctypes.c_int]),
    "cf_set_density": (ctypes.c_int, [_vp, ctypes.c_double]),
    "cf_set_warm_start": (ctypes.c_int, [_vp, ctypes.c_int]),
    "cf_set_quirks": (ctypes.c_int, [_vp, ctypes.c_uint]),
    "cf_upload": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _pd, _pd]),
    "cf_download": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _pd, _pd]),
    "cf_download_ghosted": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _ip, _ip]),
    "cf_fill_ghosts": (ctypes.c_int, [_vp]),
    "cf_advect": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int]),
    "cf_add_inputs": (ctypes.c_int, [_vp, ctypes.c_double]),
    "cf_project": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolveStats)]),
    "cf_setup": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolveStats)]),
    "cf_step": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int, ctypes.POINTER(SolverOpts),
                               ctypes.POINTER(SolveStats)]),
    "cf_steps": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.POINTER(SolverOpts),
                                ctypes.POINTER(SolveStats), ctypes.POINTER(ctypes.c_int)]),
    "cf_step_host": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int, ctypes.POINTER(SolverOpts),
                                    ctypes.POINTER(SolveStats), _dp, _dp, _dp, _dp, _dp, _dp]),
    "cf_div_norms": (ctypes.c_int, [_vp, _dp, _dp]),
    "cf_max_velocity": (ctypes.c_int, [_vp, _dp]),
    "cf_test_fail_alloc": (ctypes.c_int, [ctypes.c_int]),
    "cf_test_stall_wait": (ctypes.c_int, [_vp, ctypes.c_int]),
    "cf_test_advect_unstaged": (ctypes.c_int, [_vp, ctypes.c_int]),
    "cf_test_apply_general": (ctypes.c_int, [_vp, ctypes.c_int]),
    "cf_set_graphs": (ctypes.c_int, [_vp, ctypes.c_int]),
    "cf_test_conversions": (ctypes.c_int, [_vp, ctypes.c_int, _dp, ctypes.POINTER(ctypes.c_float), _dp]),
    "cf_test_strip_geometry": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_int, _ip, _ip, ctypes.c_int]),
    "cf_interp_points": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp]),
    "cf_trace_points": (ctypes.c_int, [_vp, ctypes.c_int, _dp, ctypes.c_double, _dp]),
    "cf_cell_velocity": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_ssize_t, ctypes.c_ssize_t]),
    "cf_launch_count": (ctypes.c_longlong, [_vp]),
    "cf_stream": (_vp, [_vp]),
    "cf_timer_start": (ctypes.c_int, [_vp]),
    "cf_timer_stop": (ctypes.c_int, [_vp, _dp]),
    "cf_profile_enable": (ctypes.c_int, [_vp, ctypes.c_int]),
    "cf_profile_read": (ctypes.c_int, [_vp, ctypes.POINTER(Profile)]),
    "cf_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(_vp)]),
    "cf_host_free": (ctypes.c_int, [_vp]),
    "cf_forward_checkpointed": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                               ctypes.POINTER(SolverOpts), ctypes.POINTER(SolveStats)]),
    "cf_backward": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "cf_div_norms_noalloc": (ctypes.c_int, [_vp, _pd, _vp, _pd, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_double, _vp, _vp]),
}

_LIB = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libcfgpu.so (raises OSError if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise OSError(
            f"{path} is missing: build it with `python -m cajitafluids_gb300.build` "
            "(the CUDA library is required; there is no CPU fallback)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib
