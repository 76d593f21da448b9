"""Python handle over the C ABI: one simulation state on one GPU.

Arrays exchanged with the context are numpy float64 arrays indexed
[gj, gi] (rows along y, x fastest), covering the owned region of a field:
quantity (ny, nx), u (ny, nx + 1 - px), v (ny + 1 - py, nx), pressure (ny, nx).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib as L

FIELDS = {"quantity": L.CF_FIELD_QUANTITY, "q": L.CF_FIELD_QUANTITY,
          "u": L.CF_FIELD_U, "v": L.CF_FIELD_V,
          "pressure": L.CF_FIELD_PRESSURE, "p": L.CF_FIELD_PRESSURE}


class CfError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{L.ERROR_NAMES.get(code, code)}: {message}")
        self.code = code


@dataclass
class SolverOptions:
    """Pressure-solver options (src/VelocityCorrector.hpp:96-106, 297-339)."""
    solver: str = "PCG"
    precon: str = "Diagonal"
    tol: float = 1.0e-6
    abs_tol: float = 0.0
    max_iter: int = 2000
    inner_tol: float = 0.0
    max_outer: int = 0

    def to_c(self) -> L.SolverOpts:
        self._keep = (self.solver.encode(), self.precon.encode())
        return L.SolverOpts(self._keep[0], self._keep[1], float(self.tol), float(self.abs_tol),
                            int(self.max_iter), float(self.inner_tol), int(self.max_outer))


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Context:
    """One grid + state on one GPU (owns all device memory)."""

    def __init__(self, nx: int, ny: int, lo=(0.0, 0.0), hi=(1.0, 1.0), periodic=(False, False),
                 precision: str = "fp64", device: int = 0):
        self.lib = L.load()
        prec = {"fp64": L.CF_PREC_FP64, "mixed": L.CF_PREC_MIXED}[precision]
        d = L.GridDesc(int(nx), int(ny), (ctypes.c_double * 2)(*lo), (ctypes.c_double * 2)(*hi),
                       (ctypes.c_int * 2)(int(bool(periodic[0])), int(bool(periodic[1]))), prec, int(device))
        h = ctypes.c_void_p()
        rc = self.lib.cf_ctx_create(ctypes.byref(d), ctypes.byref(h))
        if rc != L.CF_OK:
            raise CfError(rc, "cf_ctx_create failed")
        self.h = h
        self.nx, self.ny = int(nx), int(ny)
        self.periodic = (bool(periodic[0]), bool(periodic[1]))
        self.precision = precision

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.cf_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- helpers ------------------------------------------------------------
    def _check(self, rc: int, allow=()):
        if rc != L.CF_OK and rc not in allow:
            raise CfError(rc, self.lib.cf_last_error(self.h).decode())
        return rc

    def owned_shape(self, field) -> tuple:
        f = FIELDS[field] if isinstance(field, str) else field
        ex, ey = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.cf_owned_extent(self.h, f, ctypes.byref(ex), ctypes.byref(ey)))
        return (ey.value, ex.value)

    @property
    def dx(self) -> float:
        v = ctypes.c_double()
        self._check(self.lib.cf_cell_size(self.h, ctypes.byref(v)))
        return v.value

    # -- inputs ---------------------------------------------------------------
    def set_bc(self, types: Sequence[int]):
        arr = (ctypes.c_int * 4)(*[int(t) for t in types])
        self._check(self.lib.cf_set_bc(self.h, arr))

    def set_source(self, location, size, velocity, quantity: float, mode: int = 0):
        D2 = ctypes.c_double * 2
        self._check(self.lib.cf_set_source(self.h, D2(*location), D2(*size), D2(*velocity), float(quantity), int(mode)))

    def set_body_force(self, force, density_scaled: bool = False):
        self._check(self.lib.cf_set_body_force(self.h, (ctypes.c_double * 2)(*force), int(bool(density_scaled))))

    def set_density(self, density: float):
        self._check(self.lib.cf_set_density(self.h, float(density)))

    def set_warm_start(self, on: bool = True):
        """Start each projection from the previous pressure (extension)."""
        self._check(self.lib.cf_set_warm_start(self.h, int(bool(on))))

    def set_graphs(self, on: bool = True):
        """CUDA graphs for the pressure solve (default), or every kernel
        launched on its own (same results)."""
        self._check(self.lib.cf_set_graphs(self.h, int(bool(on))))

    def set_quirks(self, flags: int):
        self._check(self.lib.cf_set_quirks(self.h, int(flags)))

    # -- state ----------------------------------------------------------------
    def upload(self, field, arr: np.ndarray):
        f = FIELDS[field] if isinstance(field, str) else field
        shape = self.owned_shape(f)
        a = np.asarray(arr, dtype=np.float64)
        if a.shape != shape:
            raise ValueError(f"field {field}: expected shape {shape}, got {a.shape}")
        si = a.strides[1] // 8
        sj = a.strides[0] // 8
        if a.strides[1] % 8 or a.strides[0] % 8 or si <= 0 or sj <= 0:
            a = np.ascontiguousarray(a)
            si, sj = 1, a.shape[1]
        self._check(self.lib.cf_upload(self.h, f, _dptr(a), si, sj))

    def upload_strided(self, field, buf: np.ndarray, stride_i: int, stride_j: int):
        f = FIELDS[field] if isinstance(field, str) else field
        self._check(self.lib.cf_upload(self.h, f, _dptr(buf), int(stride_i), int(stride_j)))

    def download(self, field, out: Optional[np.ndarray] = None) -> np.ndarray:
        f = FIELDS[field] if isinstance(field, str) else field
        shape = self.owned_shape(f)
        if out is None:
            out = np.empty(shape, dtype=np.float64)
        assert out.shape == shape and out.dtype == np.float64 and out.flags.c_contiguous
        self._check(self.lib.cf_download(self.h, f, _dptr(out), 1, shape[1]))
        return out

    def download_strided(self, field, buf: np.ndarray, stride_i: int, stride_j: int):
        f = FIELDS[field] if isinstance(field, str) else field
        self._check(self.lib.cf_download(self.h, f, _dptr(buf), int(stride_i), int(stride_j)))

    def download_ghosted(self, field) -> np.ndarray:
        f = FIELDS[field] if isinstance(field, str) else field
        ex, ey = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.cf_download_ghosted(self.h, f, None, ctypes.byref(ex), ctypes.byref(ey)))
        out = np.empty((ey.value, ex.value), dtype=np.float64)
        self._check(self.lib.cf_download_ghosted(self.h, f, _dptr(out), ctypes.byref(ex), ctypes.byref(ey)))
        return out

    def fill_ghosts(self):
        self._check(self.lib.cf_fill_ghosts(self.h))

    # -- hot path -------------------------------------------------------------
    def advect(self, dt: float, order: int = 3):
        self._check(self.lib.cf_advect(self.h, float(dt), int(order)))

    def add_inputs(self, dt: float):
        self._check(self.lib.cf_add_inputs(self.h, float(dt)))

    def _solve_call(self, fn, *args, opts: Optional[SolverOptions] = None, raise_on_maxit=False):
        o = (opts or SolverOptions()).to_c()
        st = L.SolveStats()
        allow = () if raise_on_maxit else (L.CF_ERR_NOT_CONVERGED,)
        self._check(fn(self.h, *args, ctypes.byref(o), ctypes.byref(st)), allow=allow)
        return st.as_dict()

    def project(self, dt: float, opts: Optional[SolverOptions] = None, raise_on_maxit=False) -> dict:
        return self._solve_call(self.lib.cf_project, ctypes.c_double(dt), opts=opts, raise_on_maxit=raise_on_maxit)

    def setup(self, dt: float, opts: Optional[SolverOptions] = None, raise_on_maxit=False) -> dict:
        return self._solve_call(self.lib.cf_setup, ctypes.c_double(dt), opts=opts, raise_on_maxit=raise_on_maxit)

    def step(self, dt: float, order: int = 3, opts: Optional[SolverOptions] = None, raise_on_maxit=False) -> dict:
        return self._solve_call(self.lib.cf_step, ctypes.c_double(dt), ctypes.c_int(order), opts=opts,
                                raise_on_maxit=raise_on_maxit)

    def steps(self, nsteps: int, dt: float, order: int = 3, opts: Optional[SolverOptions] = None,
              raise_on_maxit=False) -> dict:
        """cf_steps: nsteps steps with one synchronisation; the last step's
        solve statistics plus "unconverged", the number of steps whose
        pressure solve did not converge."""
        o = (opts or SolverOptions()).to_c()
        st = L.SolveStats()
        bad = ctypes.c_int(0)
        allow = () if raise_on_maxit else (L.CF_ERR_NOT_CONVERGED,)
        self._check(self.lib.cf_steps(self.h, int(nsteps), ctypes.c_double(dt), ctypes.c_int(order), ctypes.byref(o),
                                      ctypes.byref(st), ctypes.byref(bad)), allow=allow)
        d = st.as_dict()
        d["unconverged"] = bad.value
        return d

    def step_host(self, dt: float, order: int, opts: Optional[SolverOptions], q_in, u_in, v_in, q_out=None,
                  u_out=None, v_out=None, raise_on_maxit=False) -> dict:
        """cf_step_host: upload q, u, v, one step, download into the outputs
        (owned shapes, C order, float64; page-locked arrays copy fastest)."""
        shapes = (self.owned_shape("q"), self.owned_shape("u"), self.owned_shape("v"))
        ins = []
        for a, shp in zip((q_in, u_in, v_in), shapes):
            a = np.ascontiguousarray(a, dtype=np.float64)
            if a.shape != shp:
                raise ValueError(f"expected shape {shp}, got {a.shape}")
            ins.append(a)
        outs = []
        for a, shp in zip((q_out, u_out, v_out), shapes):
            if a is not None and (a.shape != shp or a.dtype != np.float64 or not a.flags.c_contiguous):
                raise ValueError(f"output must be a C-contiguous float64 array of shape {shp}")
            outs.append(_dptr(a) if a is not None else None)
        o = (opts or SolverOptions()).to_c()
        st = L.SolveStats()
        allow = () if raise_on_maxit else (L.CF_ERR_NOT_CONVERGED,)
        self._check(self.lib.cf_step_host(self.h, ctypes.c_double(dt), ctypes.c_int(order), ctypes.byref(o),
                                          ctypes.byref(st), *[_dptr(a) for a in ins], *outs), allow=allow)
        return st.as_dict()

    # -- adjoint ----------------------------------------------------------------
    def forward_checkpointed(self, nsteps: int, ckpt_every: int, dt: float, order: int = 3,
                             opts: Optional[SolverOptions] = None) -> dict:
        o = (opts or SolverOptions()).to_c()
        st = L.SolveStats()
        self._check(self.lib.cf_forward_checkpointed(self.h, int(nsteps), int(ckpt_every), float(dt), int(order),
                                                     ctypes.byref(o), ctypes.byref(st)))
        return st.as_dict()

    def backward(self, dq_T: np.ndarray, du_T: Optional[np.ndarray] = None,
                 dv_T: Optional[np.ndarray] = None) -> dict:
        def arg(a, field):
            if a is None:
                return None, None
            a = np.ascontiguousarray(a, dtype=np.float64)
            assert a.shape == self.owned_shape(field)
            return a, _dptr(a)
        keep = [arg(dq_T, "q"), arg(du_T, "u"), arg(dv_T, "v")]
        out = {f: np.empty(self.owned_shape(f)) for f in ("q", "u", "v")}
        rate = ctypes.c_double()
        self._check(self.lib.cf_backward(self.h, keep[0][1], keep[1][1], keep[2][1], _dptr(out["q"]),
                                         _dptr(out["u"]), _dptr(out["v"]), ctypes.byref(rate)))
        out["rate"] = rate.value
        return out

    def div_norms(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.cf_div_norms(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def test_conversions(self, d: np.ndarray):
        """The device's integer-pipe FP64 -> FP32 and FP32 -> FP64 conversions of d."""
        d = np.ascontiguousarray(d, dtype=np.float64).ravel()
        f = np.empty(d.size, dtype=np.float32)
        w = np.empty(d.size, dtype=np.float64)
        self._check(self.lib.cf_test_conversions(self.h, d.size, d.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                 f.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                 w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return f, w

    def max_velocity(self) -> float:
        a = ctypes.c_double()
        self._check(self.lib.cf_max_velocity(self.h, ctypes.byref(a)))
        return a.value

    def interp_points(self, field, order: int, xy: np.ndarray) -> np.ndarray:
        f = FIELDS[field] if isinstance(field, str) else field
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        out = np.empty(xy.shape[0], dtype=np.float64)
        self._check(self.lib.cf_interp_points(self.h, f, int(order), xy.shape[0], _dptr(xy), _dptr(out)))
        return out

    def trace_points(self, xy: np.ndarray, dt: float) -> np.ndarray:
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        out = np.empty_like(xy)
        self._check(self.lib.cf_trace_points(self.h, xy.shape[0], _dptr(xy), float(dt), _dptr(out)))
        return out

    def cell_velocity(self):
        """Cell-centred (linear) velocity of the current state, as SiloWriter
        writes it: two (ny, nx) arrays."""
        ny, nx = self.owned_shape("q")
        uc = np.empty((ny, nx))
        vc = np.empty((ny, nx))
        self._check(self.lib.cf_cell_velocity(self.h, _dptr(uc), _dptr(vc), 1, nx))
        return uc, vc

    @property
    def launches(self) -> int:
        return int(self.lib.cf_launch_count(self.h))

    @property
    def stream(self) -> int:
        return int(self.lib.cf_stream(self.h) or 0)

    def timer_start(self):
        self._check(self.lib.cf_timer_start(self.h))

    def timer_stop(self) -> float:
        ms = ctypes.c_double()
        self._check(self.lib.cf_timer_stop(self.h, ctypes.byref(ms)))
        return ms.value

    def profile_enable(self, on: bool = True):
        self._check(self.lib.cf_profile_enable(self.h, int(bool(on))))

    def profile_read(self) -> dict:
        p = L.Profile()
        self._check(self.lib.cf_profile_read(self.h, ctypes.byref(p)))
        return p.as_dict()


class PinnedArray:
    """Page-locked host buffer viewed as a float64 numpy array."""

    def __init__(self, shape):
        self.lib = L.load()
        n = int(np.prod(shape))
        ptr = ctypes.c_void_p()
        rc = self.lib.cf_host_alloc(n * 8, ctypes.byref(ptr))
        if rc != L.CF_OK:
            raise CfError(rc, "cf_host_alloc failed")
        self.ptr = ptr
        buf = (ctypes.c_double * n).from_address(ptr.value)
        self.array = np.frombuffer(buf, dtype=np.float64).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            self.lib.cf_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
