"""CPU oracle of the cajitafluids hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
this package, as the checker or the timed CPU baseline; the product
(cajitafluids_gb300) never imports it.  Parity status: unpinned against the
reference's numerics (the reference cannot be built here); the geometry and
state conventions are pinned against the reference's own Mesh and
ProblemManager tests.  See cf_oracle.c for the reference citations.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .build import build_oracle

Q, U, V, P, RHS = 0, 1, 2, 3, 4
_FIELDS = {"quantity": Q, "q": Q, "u": U, "v": V, "pressure": P, "p": P, "rhs": RHS}


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("lo", ctypes.c_double * 2), ("hi", ctypes.c_double * 2),
        ("periodic", ctypes.c_int * 2), ("bc_type", ctypes.c_int * 4),
        ("src_bbox", ctypes.c_double * 4), ("src_quantity", ctypes.c_double),
        ("src_velocity", ctypes.c_double * 2), ("src_mode", ctypes.c_int),
        ("body_force", ctypes.c_double * 2), ("body_density_scaled", ctypes.c_int),
        ("density", ctypes.c_double), ("quirks", ctypes.c_uint), ("precon_none", ctypes.c_int),
        ("precon_mg", ctypes.c_int), ("warm_start", ctypes.c_int),
    ]


class OrcStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("status", ctypes.c_int), ("bb", ctypes.c_double),
                ("rr", ctypes.c_double), ("div_l2", ctypes.c_double), ("div_linf", ctypes.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_oracle())
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        vp = ctypes.c_void_p
        sig = {
            "orc_create": (vp, [ctypes.POINTER(OrcParams), ctypes.c_char_p, ctypes.c_int]),
            "orc_destroy": (None, [vp]),
            "orc_owned_extent": (ctypes.c_int, [vp, ctypes.c_int, ip, ip]),
            "orc_ghosted_extent": (ctypes.c_int, [vp, ctypes.c_int, ip, ip]),
            "orc_set_field": (ctypes.c_int, [vp, ctypes.c_int, dp]),
            "orc_get_field": (ctypes.c_int, [vp, ctypes.c_int, dp]),
            "orc_get_ghosted": (ctypes.c_int, [vp, ctypes.c_int, dp]),
            "orc_set_ghosted": (ctypes.c_int, [vp, ctypes.c_int, dp]),
            "orc_fill_ghosts": (None, [vp]),
            "orc_advect_step": (None, [vp, ctypes.c_double, ctypes.c_int]),
            "orc_add_inputs": (None, [vp, ctypes.c_double]),
            "orc_project": (ctypes.c_int, [vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                           ctypes.POINTER(OrcStats)]),
            "orc_step": (ctypes.c_int, [vp, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, ctypes.POINTER(OrcStats)]),
            "orc_div_norms": (None, [vp, dp, dp]),
            "orc_sample": (None, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp]),
            "orc_trace": (None, [vp, ctypes.c_int, dp, ctypes.c_double, dp]),
            "orc_matvec": (None, [vp, ctypes.c_double, dp, dp]),
            "orc_canonical_dot": (ctypes.c_double, [ctypes.c_int, ctypes.c_int, dp, dp]),
            "orc_mg_apply": (ctypes.c_int, [vp, ctypes.c_double, dp, dp]),
            "orc_threads": (ctypes.c_int, []),
        }
        for k, (r, a) in sig.items():
            f = getattr(_lib, k)
            f.restype = r
            f.argtypes = a
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def canonical_dot(a: np.ndarray, b: np.ndarray) -> float:
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    ny, nx = a.shape
    return lib().orc_canonical_dot(nx, ny, _dp(a), _dp(b))


def threads() -> int:
    return lib().orc_threads()


class Oracle:
    """FP64 CPU restatement of one cajitafluids simulation state."""

    def __init__(self, nx, ny, lo=(0.0, 0.0), hi=(1.0, 1.0), periodic=(False, False), bc=(0, 0, 0, 0),
                 source=None, source_mode=0, body=(0.0, 0.0), body_density_scaled=False, density=1.0,
                 quirks=0, precon_none=False, precon_mg=False, warm_start=False):
        p = OrcParams()
        p.nx, p.ny = int(nx), int(ny)
        p.lo[:] = list(lo)
        p.hi[:] = list(hi)
        p.periodic[:] = [int(bool(periodic[0])), int(bool(periodic[1]))]
        p.bc_type[:] = [int(b) for b in bc]
        if source is not None:
            (x0, y0), (w, h), vel, qty = source
            p.src_bbox[:] = [x0, y0, x0 + w, y0 + h]
            p.src_velocity[:] = list(vel)
            p.src_quantity = float(qty)
        p.src_mode = int(source_mode)
        p.body_force[:] = list(body)
        p.body_density_scaled = int(bool(body_density_scaled))
        p.density = float(density)
        p.quirks = int(quirks)
        p.precon_none = int(bool(precon_none))
        p.precon_mg = int(bool(precon_mg))
        p.warm_start = int(bool(warm_start))
        err = ctypes.create_string_buffer(256)
        self.lib = lib()
        self.h = self.lib.orc_create(ctypes.byref(p), err, 256)
        if not self.h:
            raise ValueError(err.value.decode())
        self.nx, self.ny = int(nx), int(ny)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def shape(self, field):
        f = _FIELDS[field] if isinstance(field, str) else field
        ex, ey = ctypes.c_int(), ctypes.c_int()
        self.lib.orc_owned_extent(self.h, f, ctypes.byref(ex), ctypes.byref(ey))
        return (ey.value, ex.value)

    def set(self, field, arr):
        f = _FIELDS[field] if isinstance(field, str) else field
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == self.shape(f), (a.shape, self.shape(f))
        self.lib.orc_set_field(self.h, f, _dp(a))

    def get(self, field):
        f = _FIELDS[field] if isinstance(field, str) else field
        out = np.empty(self.shape(f), dtype=np.float64)
        self.lib.orc_get_field(self.h, f, _dp(out))
        return out

    def get_ghosted(self, field):
        f = _FIELDS[field] if isinstance(field, str) else field
        ex, ey = ctypes.c_int(), ctypes.c_int()
        self.lib.orc_ghosted_extent(self.h, f, ctypes.byref(ex), ctypes.byref(ey))
        out = np.empty((ey.value, ex.value), dtype=np.float64)
        self.lib.orc_get_ghosted(self.h, f, _dp(out))
        return out

    def set_ghosted(self, field, arr):
        f = _FIELDS[field] if isinstance(field, str) else field
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self.lib.orc_set_ghosted(self.h, f, _dp(a))

    def fill_ghosts(self):
        self.lib.orc_fill_ghosts(self.h)

    def advect(self, dt, order=3):
        self.lib.orc_advect_step(self.h, float(dt), int(order))

    def add_inputs(self, dt):
        self.lib.orc_add_inputs(self.h, float(dt))

    def project(self, dt, tol=1e-6, abs_tol=0.0, max_iter=2000):
        st = OrcStats()
        self.lib.orc_project(self.h, float(dt), float(tol), float(abs_tol), int(max_iter), ctypes.byref(st))
        return {k: getattr(st, k) for k, _ in OrcStats._fields_}

    def setup(self, dt, tol=1e-6, abs_tol=0.0, max_iter=2000):
        self.add_inputs(dt)
        return self.project(dt, tol, abs_tol, max_iter)

    def step(self, dt, order=3, tol=1e-6, abs_tol=0.0, max_iter=2000):
        st = OrcStats()
        self.lib.orc_step(self.h, float(dt), int(order), float(tol), float(abs_tol), int(max_iter),
                          ctypes.byref(st))
        return {k: getattr(st, k) for k, _ in OrcStats._fields_}

    def div_norms(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self.lib.orc_div_norms(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def sample(self, field, order, xy):
        f = _FIELDS[field] if isinstance(field, str) else field
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        out = np.empty(xy.shape[0])
        self.lib.orc_sample(self.h, f, int(order), xy.shape[0], _dp(xy), _dp(out))
        return out

    def trace(self, xy, dt):
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        out = np.empty_like(xy)
        self.lib.orc_trace(self.h, xy.shape[0], _dp(xy), float(dt), _dp(out))
        return out

    def mg_apply(self, dt, r):
        """One multigrid V-cycle applied to r; returns (z, levels)."""
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.empty_like(r)
        nlev = self.lib.orc_mg_apply(self.h, float(dt), _dp(r), _dp(z))
        return z, nlev

    def matvec(self, dt, p):
        p = np.ascontiguousarray(p, dtype=np.float64)
        out = np.empty_like(p)
        self.lib.orc_matvec(self.h, float(dt), _dp(p), _dp(out))
        return out
