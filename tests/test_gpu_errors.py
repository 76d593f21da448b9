"""Error behaviour of the C ABI: every failure is a status code, the context
stays usable, and nothing is injected on the device (faults are made on the
host: bad arguments, NaN inputs, tight iteration limits)."""
import ctypes

import numpy as np
import pytest

from cajitafluids_gb300 import CfError, Context, SolverOptions
from cajitafluids_gb300 import _lib as L
from helpers import load_state, make_pair, opts, random_state

pytestmark = pytest.mark.gpu


def test_invalid_arguments(built):
    lib = L.load()
    h = ctypes.c_void_p()
    assert lib.cf_ctx_create(None, ctypes.byref(h)) == L.CF_ERR_INVALID
    d = L.GridDesc(0, 8, (ctypes.c_double * 2)(0, 0), (ctypes.c_double * 2)(1, 1), (ctypes.c_int * 2)(0, 0), 0, 0)
    assert lib.cf_ctx_create(ctypes.byref(d), ctypes.byref(h)) == L.CF_ERR_INVALID
    # extent not divisible by the uniform cell size (src/Mesh.hpp:49-64)
    d = L.GridDesc(8, 8, (ctypes.c_double * 2)(0, 0), (ctypes.c_double * 2)(1, 2), (ctypes.c_int * 2)(0, 0), 0, 0)
    assert lib.cf_ctx_create(ctypes.byref(d), ctypes.byref(h)) == L.CF_ERR_MESH
    assert lib.cf_step(None, 0.1, 3, None, None) == L.CF_ERR_INVALID
    c = Context(8, 8)
    with pytest.raises(CfError) as e:
        c.advect(0.1, order=2)
    assert e.value.code == L.CF_ERR_INVALID
    with pytest.raises(CfError):
        c.set_bc((0, 0, 7, 0))
    with pytest.raises(CfError):
        c.set_density(-1.0)
    with pytest.raises(CfError):
        c.step(-1.0)
    with pytest.raises(ValueError):
        c.upload("u", np.zeros((8, 8)))   # u is (8, 9)
    assert lib.cf_upload(c.h, 1, None, 1, 9) == L.CF_ERR_INVALID
    # the context still works
    c.upload("u", np.ones((8, 9)))
    assert c.download("u").sum() == 72.0


@pytest.mark.parametrize("solver,precon", [("GMRES", "Diagonal"), ("PCG", "Euclid"), ("PCG", "ParaSails"),
                                            ("BiCGSTAB", "None")])
def test_unsupported_solvers(built, solver, precon):
    c = Context(16, 16)
    with pytest.raises(CfError) as e:
        c.project(0.01, SolverOptions(solver=solver, precon=precon))
    assert e.value.code == L.CF_ERR_UNSUPPORTED
    assert "not implemented" in str(e.value)


def test_reference_solver_name(built):
    o, c = make_pair(20, 20)
    rng = np.random.default_rng(0)
    load_state(o, c, random_state(o, rng))
    s = c.project(0.01, SolverOptions(solver="Reference", precon="PFMG", tol=1e-8, max_iter=5000))
    so = o.project(0.01, tol=1e-8, max_iter=5000)
    assert s["iterations"] == so["iterations"]


def test_max_iter_is_reported_and_state_consistent(built):
    o, c = make_pair(32, 32)
    rng = np.random.default_rng(1)
    load_state(o, c, random_state(o, rng))
    with pytest.raises(CfError) as e:
        c.project(0.01, opts(tol=1e-12, max_iter=3), raise_on_maxit=True)
    assert e.value.code == L.CF_ERR_NOT_CONVERGED
    o2, c2 = make_pair(32, 32)
    load_state(o2, c2, random_state(o2, np.random.default_rng(1)))
    s = c2.project(0.01, opts(tol=1e-12, max_iter=3))
    so = o2.project(0.01, tol=1e-12, max_iter=3)
    assert s["status"] == L.CF_SOLVE_MAX_ITER and so["status"] == 1
    assert s["iterations"] == 3
    assert np.array_equal(o2.get("p"), c2.download("p"))
    assert np.array_equal(o2.get("u"), c2.download("u"))


def test_zero_state_needs_no_iterations(built):
    o, c = make_pair(24, 24)
    s = c.project(0.01, opts())
    assert s["iterations"] == 0 and s["status"] == 0 and s["b_norm"] == 0.0
    assert not c.download("p").any()


def test_nan_input_gives_numeric_error(built):
    c = Context(16, 16)
    u = np.zeros((16, 17))
    u[5, 5] = np.nan
    c.upload("u", u)
    with pytest.raises(CfError) as e:
        c.project(0.01, opts())
    assert e.value.code == L.CF_ERR_NUMERIC
    # still usable afterwards
    c.upload("u", np.zeros((16, 17)))
    assert c.project(0.01, opts())["status"] == 0


def test_strided_layouts(built):
    """Kokkos LayoutLeft / LayoutRight host mirrors go through the strides."""
    rng = np.random.default_rng(3)
    c = Context(10, 7, hi=(1.0, 0.7))
    u = rng.standard_normal((7, 11))
    # LayoutRight-like: i slowest (buf[i, j])
    buf = np.ascontiguousarray(u.T)
    c.upload_strided("u", buf, stride_i=7, stride_j=1)
    assert np.array_equal(c.download("u"), u)
    out = np.zeros_like(buf)
    c.download_strided("u", out, stride_i=7, stride_j=1)
    assert np.array_equal(out, buf)
    # padded rows
    big = np.zeros((7, 16))
    big[:, :11] = u
    c.upload_strided("u", big, 1, 16)
    assert np.array_equal(c.download("u"), u)


def test_mixed_context_roundtrip(built):
    c = Context(16, 12, hi=(1.0, 0.75), precision="mixed")
    q = np.random.default_rng(0).uniform(0, 1, (12, 16))
    c.upload("q", q)
    assert np.array_equal(c.download("q"), q.astype(np.float32).astype(np.float64))
    with pytest.raises(CfError) as e:
        c.interp_points("q", 3, np.zeros((1, 2)))
    assert e.value.code == L.CF_ERR_UNSUPPORTED


@pytest.mark.parametrize("precon", ["Diagonal", "PFMG"])
@pytest.mark.parametrize("graphs", [True, False])
def test_device_wait_timeout_is_reported_and_context_usable(built, precon, graphs):
    """The mixed inner CG's bounded mbarrier waits: with the test hook one
    CTA's first tile wait is on a barrier that nothing arrives on, so it runs
    out (no GPU fault: the CTA records the timeout, waits for its own copies
    and returns).  The projection returns CF_ERR_TIMEOUT; with the hook off
    the same context projects the same state to the same bits as a fresh
    context."""
    lib = L.load()
    n = 256
    rng = np.random.default_rng(8)
    o, a = make_pair(n, n, precision="mixed")
    b = make_pair(n, n, precision="mixed")[1]
    a.set_graphs(graphs)
    # random face velocities (wall-normal ones zero): a consistent, far from
    # divergence-free right-hand side
    st = random_state(o, rng, scale=0.1)
    so = opts(tol=1e-8, max_iter=5000, precon=precon)
    load_state(o, a, st)
    assert lib.cf_test_stall_wait(a.h, 1) == L.CF_OK
    try:
        with pytest.raises(CfError) as e:
            a.project(0.002, so, raise_on_maxit=True)
        assert e.value.code == L.CF_ERR_TIMEOUT
        assert "timed out" in str(e.value)
    finally:
        lib.cf_test_stall_wait(a.h, 0)
    for f in ("q", "u", "v"):
        a.upload(f, st[f])
        b.upload(f, st[f])
    sa = a.project(0.002, so, raise_on_maxit=True)
    sb = b.project(0.002, so, raise_on_maxit=True)
    assert sa["iterations"] == sb["iterations"] and sa["div_l2"] == sb["div_l2"]
    for f in ("p", "u", "v"):
        assert np.array_equal(a.download(f), b.download(f)), f
