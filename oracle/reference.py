"""The reference's own step, run on the host -- TEST INFRASTRUCTURE ONLY.

Wraps oracle/_ref/libcfref.so (built by oracle.build.build_reference from
the reference's unchanged src/*.hpp and the stand-ins in oracle/refshim).
Used by tests/test_reference_pin.py to pin the oracle, and by
tests/golden/make_golden.py to write fixtures that carry the reference's
own results.  Only available where the reference's sources are present.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .build import build_reference


class RefParams(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("lo", ctypes.c_double * 2),
                ("hi", ctypes.c_double * 2), ("bc", ctypes.c_int * 4), ("src_loc", ctypes.c_double * 2),
                ("src_size", ctypes.c_double * 2), ("src_vel", ctypes.c_double * 2), ("src_q", ctypes.c_double),
                ("force", ctypes.c_double * 2), ("density", ctypes.c_double), ("dt", ctypes.c_double)]


_lib = None


def available() -> bool:
    return build_reference() is not None


def lib():
    global _lib
    if _lib is None:
        path = build_reference()
        if path is None:
            raise RuntimeError("the reference's sources are not on this machine")
        _lib = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        _lib.cfref_run.restype = ctypes.c_int
        _lib.cfref_run.argtypes = [ctypes.POINTER(RefParams), dp, dp, dp, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_double, ctypes.c_int, dp, dp, dp, dp, ip, ip, ctypes.c_int, ip, ip,
                                   ctypes.c_char_p, ctypes.c_int]
        _lib.cfref_functor.restype = ctypes.c_int
        _lib.cfref_functor.argtypes = [ctypes.POINTER(RefParams), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_double, dp]
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def params(nx, ny, lo=(0.0, 0.0), hi=(1.0, 1.0), bc=(0, 0, 0, 0), source=None, body=(0.0, 0.0), density=1.0,
           dt=1e-3) -> RefParams:
    """source = (location, size, velocity, quantity) as InflowSource<2>
    takes them (src/InflowSource.hpp:80-90); None = an empty box."""
    if source is None:
        source = ((0.0, 0.0), (0.0, 0.0), (0.0, 0.0), 0.0)
    D2 = ctypes.c_double * 2
    return RefParams(int(nx), int(ny), D2(*lo), D2(*hi), (ctypes.c_int * 4)(*bc), D2(*source[0]), D2(*source[1]),
                     D2(*source[2]), float(source[3]), D2(*body), float(density), float(dt))


def run(prm: RefParams, q0=None, u0=None, v0=None, steps=0, t_final=None, write_freq=1):
    """setup() + `steps` step() calls (t_final None), or solve(t_final,
    write_freq), through createSolver("serial", ...) with the "Reference"
    solver.  Returns q, u, v, p (owned, row-major), the iterations and
    status of every pressure solve, and the SiloWriter write count."""
    L = lib()
    nx, ny = prm.nx, prm.ny
    ins = []
    for a, shp in ((q0, (ny, nx)), (u0, (ny, nx + 1)), (v0, (ny + 1, nx))):
        if a is not None:
            a = np.ascontiguousarray(a, dtype=np.float64)
            assert a.shape == shp, (a.shape, shp)
        ins.append(a)
    q = np.empty((ny, nx))
    u = np.empty((ny, nx + 1))
    v = np.empty((ny + 1, nx))
    p = np.zeros((ny, nx))
    cap = 100000
    its = np.zeros(cap, dtype=np.int32)
    sts = np.zeros(cap, dtype=np.int32)
    nsolves = ctypes.c_int()
    writes = ctypes.c_int()
    err = ctypes.create_string_buffer(512)
    mode = 0 if t_final is None else 1
    rc = L.cfref_run(ctypes.byref(prm), *[_dp(a) for a in ins], mode, int(steps),
                     float(t_final or 0.0), int(write_freq), _dp(q), _dp(u), _dp(v), _dp(p),
                     its.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                     sts.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), cap, ctypes.byref(nsolves),
                     ctypes.byref(writes), err, len(err))
    if rc != 0:
        raise RuntimeError(err.value.decode())
    n = nsolves.value
    return {"q": q, "u": u, "v": v, "p": p, "iterations": its[:n].copy(), "status": sts[:n].copy(),
            "writes": writes.value}


FUNCTOR_KINDS = {"cell_inflow": 0, "iface_inflow": 1, "jface_inflow": 2, "iface_body": 3, "jface_body": 4,
                 "iface_bc": 5, "jface_bc": 6, "build_matrix": 7}


def functor(prm: RefParams, kind: str, gi=0, gj=0, x=0.0, y=0.0, value=0.0, scale=0.0):
    """One call of the reference's InflowSource / BodyForce / BoundaryCondition
    functors on one entity value (build_matrix: the five entries
    initializeMatrixValues sets, then build_matrix)."""
    k = FUNCTOR_KINDS[kind]
    if k == 7:
        buf = np.array([4.0 * scale, -1.0 * scale, -1.0 * scale, -1.0 * scale, -1.0 * scale, scale])
    else:
        buf = np.array([float(value)])
    rc = lib().cfref_functor(ctypes.byref(prm), k, int(gi), int(gj), float(x), float(y), _dp(buf))
    assert rc == 0
    return buf[:5].copy() if k == 7 else float(buf[0])
