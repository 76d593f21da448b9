"""cf_div_norms_noalloc: divergence norms for callers that cannot allocate.

Some users of this library own their velocity arrays on the device and are
not allowed to allocate device memory where they want the norm (their memory
belongs to their own pool allocator, or the call sits in a latency-critical
loop where cudaMalloc would synchronise the device).  The allocation-free
entry point takes their device arrays directly and keeps its reduction
scratch in a fixed array inside the library.  It must give what the
context-based cf_div_norms gives -- bit for bit, the tolerance of the other
FP64 parity tests -- on consecutive calls that reuse the shared scratch.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from cajitafluids_gb300 import Context
from cajitafluids_gb300 import _lib as L

pytestmark = pytest.mark.gpu


class _Rt:
    """The few CUDA runtime calls the test needs to stage caller-owned arrays."""

    def __init__(self):
        self.rt = None
        for name in ("libcudart.so.13", "libcudart.so", "libcudart.so.12"):
            try:
                self.rt = ctypes.CDLL(name)
                break
            except OSError:
                continue
        assert self.rt is not None, "libcudart not found"
        self.ptrs = []

    def put(self, a: np.ndarray) -> int:
        a = np.ascontiguousarray(a, dtype=np.float64)
        p = ctypes.c_void_p()
        assert self.rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(max(a.nbytes, 16))) == 0
        self.ptrs.append(p.value)
        assert self.rt.cudaMemcpy(ctypes.c_void_p(p.value), a.ctypes.data_as(ctypes.c_void_p),
                                  ctypes.c_size_t(a.nbytes), 1) == 0  # host to device
        return p.value

    def get(self, ptr: int, n: int) -> np.ndarray:
        out = np.empty(n, dtype=np.float64)
        assert self.rt.cudaDeviceSynchronize() == 0
        assert self.rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(ptr),
                                  ctypes.c_size_t(out.nbytes), 2) == 0  # device to host
        return out

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFree(ctypes.c_void_p(p))
        self.ptrs = []


def _noalloc(lib, du, upitch, dv, vpitch, nx, ny, per, dx, out):
    return lib.cf_div_norms_noalloc(ctypes.c_void_p(du), upitch, ctypes.c_void_p(dv), vpitch, nx, ny, int(per[0]),
                                    int(per[1]), dx, ctypes.c_void_p(out), None)


@pytest.mark.parametrize("nx,ny,per", [(200, 150, (False, False)), (128, 128, (True, True)),
                                       (97, 64, (True, False))])
def test_noalloc_matches_context_entry_point(built, nx, ny, per):
    lib = L.load()
    rt = _Rt()
    try:
        c = Context(nx, ny, hi=(1.0, ny / nx), periodic=per)
        rng = np.random.default_rng(nx + ny)
        u = rng.standard_normal(c.owned_shape("u"))
        v = rng.standard_normal(c.owned_shape("v"))
        out = rt.put(np.zeros(2))
        for call in range(2):
            if call == 1:  # second call in a row, on different data
                u = u * -0.5 + 0.25
                v = np.roll(v, 3, axis=1)
            c.upload("u", u)
            c.upload("v", v)
            ref = c.div_norms()
            du, dv = rt.put(u), rt.put(v)
            rc = _noalloc(lib, du, u.shape[1], dv, v.shape[1], nx, ny, per, c.dx, out)
            assert rc == L.CF_OK
            got = rt.get(out, 2)
            assert got[0] == ref[0] and got[1] == ref[1], (call, got, ref)
        c.close()
    finally:
        rt.free()


def test_noalloc_rejects_grids_beyond_its_scratch(built):
    lib = L.load()
    rt = _Rt()
    try:
        dummy = rt.put(np.zeros(4))
        nx, ny = 64 * 512, 16 * 129   # 66048 units > CF_NOALLOC_MAX_UNITS
        assert (nx // 64) * (ny // 16) > L.CF_NOALLOC_MAX_UNITS
        rc = _noalloc(lib, dummy, nx + 1, dummy, nx, nx, ny, (False, False), 1.0 / nx, dummy)
        assert rc == L.CF_ERR_TOO_LARGE
        assert _noalloc(lib, 0, 10, dummy, 10, 9, 9, (False, False), 0.1, dummy) == L.CF_ERR_INVALID
    finally:
        rt.free()
