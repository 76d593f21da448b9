"""Committed golden fixtures (tests/golden/*.npz, made by make_golden.py).

reference_*.npz hold the reference's own results (its src/*.hpp compiled
unchanged against the stand-ins in oracle/refshim); the others are oracle
outputs.
CPU: the oracle reproduces all of them bit for bit (it is deterministic and
contraction-free, so x86 and Arm give the same bits).
GPU: the FP64 CUDA path reproduces them bit for bit through the C ABI.
"""
import os

import numpy as np
import pytest

from oracle import Oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INFLOW = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def _run_config0(sim, g, gpu):
    n = int(g["n"])
    dt = float(g["dt"])
    its = []
    if gpu:
        from cajitafluids_gb300 import SolverOptions
        o = SolverOptions(tol=float(g["tol"]), max_iter=20000)
        its.append(sim.setup(dt, o)["iterations"])
        for _ in range(int(g["steps"])):
            its.append(sim.step(dt, int(g["order"]), o)["iterations"])
    else:
        its.append(sim.setup(dt, tol=float(g["tol"]), max_iter=20000)["iterations"])
        for _ in range(int(g["steps"])):
            its.append(sim.step(dt, int(g["order"]), tol=float(g["tol"]), max_iter=20000)["iterations"])
    return np.array(its)


def test_oracle_reproduces_config0_fixture(built):
    g = _load("config0_32.npz")
    n = int(g["n"])
    o = Oracle(n, n, source=INFLOW, density=0.1)
    its = _run_config0(o, g, gpu=False)
    assert np.array_equal(its, g["iterations"])
    for f in ("q", "u", "v", "p"):
        assert np.array_equal(o.get(f), g[f]), f


def test_oracle_reproduces_periodic_fixture(built):
    g = _load("periodic_spectral_32.npz")
    n = int(g["n"])
    o = Oracle(n, n, periodic=(True, True), density=0.1)
    for f in ("q", "u", "v"):
        o.set(f, g[f + "0"])
    its = [o.step(float(g["dt"]), 3, tol=0.0, abs_tol=float(g["abs_tol"]), max_iter=20000)["iterations"]
           for _ in range(int(g["steps"]))]
    assert np.array_equal(its, g["iterations"])
    for f in ("q", "u", "v", "p"):
        assert np.array_equal(o.get(f), g[f]), f


def test_oracle_reproduces_walls_buoyancy_mg_fixture(built):
    """Walls, inflow, gravity scaled by the quantity, cubic values, PCG with
    the multigrid preconditioner: iterations, divergence norms and fields."""
    g = _load("walls_buoyancy_mg_48.npz")
    n = int(g["n"])
    dt, tol = float(g["dt"]), float(g["tol"])
    o = Oracle(n, n, source=INFLOW, body=(0.0, -9.8), body_density_scaled=True, density=0.1, precon_mg=True)
    st = [o.setup(dt, tol=tol, max_iter=500)]
    st += [o.step(dt, int(g["order"]), tol=tol, max_iter=500) for _ in range(int(g["steps"]))]
    assert np.array_equal([s["iterations"] for s in st], g["iterations"])
    assert np.array_equal([s["div_l2"] for s in st], g["div_l2"])
    for f in ("q", "u", "v", "p"):
        assert np.array_equal(o.get(f), g[f]), f


def test_oracle_reproduces_interpolation_fixture(built):
    g = _load("interp_kat_24.npz")
    n = int(g["n"])
    o = Oracle(n, n, periodic=(True, True))
    for f in ("q", "u", "v"):
        o.set(f, g[f])
    o.fill_ghosts()
    for f in ("q", "u", "v"):
        for order in (1, 3):
            assert np.array_equal(o.sample(f, order, g["xy"]), g[f"{f}_o{order}"])
    assert np.array_equal(o.trace(g["xy"], 0.01), g["trace"])


@pytest.mark.gpu
def test_gpu_reproduces_config0_fixture(built):
    from cajitafluids_gb300 import Context
    g = _load("config0_32.npz")
    n = int(g["n"])
    c = Context(n, n)
    c.set_source(*INFLOW)
    c.set_density(0.1)
    its = _run_config0(c, g, gpu=True)
    assert np.array_equal(its, g["iterations"])
    for f in ("q", "u", "v", "p"):
        assert np.array_equal(c.download(f), g[f]), f


@pytest.mark.gpu
def test_gpu_reproduces_periodic_fixture(built):
    from cajitafluids_gb300 import Context, SolverOptions
    g = _load("periodic_spectral_32.npz")
    n = int(g["n"])
    c = Context(n, n, periodic=(True, True))
    c.set_density(0.1)
    for f in ("q", "u", "v"):
        c.upload(f, g[f + "0"])
    o = SolverOptions(tol=0.0, abs_tol=float(g["abs_tol"]), max_iter=20000)
    its = [c.step(float(g["dt"]), 3, o)["iterations"] for _ in range(int(g["steps"]))]
    assert np.array_equal(its, g["iterations"])
    for f in ("q", "u", "v", "p"):
        assert np.array_equal(c.download(f), g[f]), f


@pytest.mark.gpu
def test_gpu_reproduces_interpolation_fixture(built):
    from cajitafluids_gb300 import Context
    g = _load("interp_kat_24.npz")
    n = int(g["n"])
    c = Context(n, n, periodic=(True, True))
    for f in ("q", "u", "v"):
        c.upload(f, g[f])
    c.fill_ghosts()
    for f in ("q", "u", "v"):
        for order in (1, 3):
            assert np.array_equal(c.interp_points(f, order, g["xy"]), g[f"{f}_o{order}"])
    assert np.array_equal(c.trace_points(g["xy"], 0.01), g["trace"])


@pytest.mark.gpu
def test_gpu_reproduces_walls_buoyancy_mg_fixture(built):
    """Walls, inflow, gravity scaled by the quantity, cubic values and the
    multigrid-preconditioned CG on the GPU: iterations, divergence norms and
    fields bit for bit."""
    from cajitafluids_gb300 import Context, SolverOptions
    g = _load("walls_buoyancy_mg_48.npz")
    n = int(g["n"])
    dt, tol = float(g["dt"]), float(g["tol"])
    c = Context(n, n)
    c.set_source(*INFLOW)
    c.set_body_force((0.0, -9.8), True)
    c.set_density(0.1)
    o = SolverOptions(tol=tol, max_iter=500, precon="PFMG")
    st = [c.setup(dt, o)]
    st += [c.step(dt, int(g["order"]), o) for _ in range(int(g["steps"]))]
    assert np.array_equal([s["iterations"] for s in st], g["iterations"])
    assert np.array_equal([s["div_l2"] for s in st], g["div_l2"])
    for f in ("q", "u", "v", "p"):
        assert np.array_equal(c.download(f), g[f]), f


# ---- fixtures written by the reference's own code ----------------------------
# The reference hard-codes cubic values and a Jacobi-preconditioned CG with
# tolerance 1e-6 and 2000 iterations (src/TimeIntegrator.hpp:112-113,
# src/VelocityCorrector.hpp:103-104, 158-180).
REF_FIXTURES = ("reference_config0_64.npz", "reference_random_walls_gravity_40.npz")


def _ref_setup(g):
    bc = tuple(int(b) for b in g["bc"]) if "bc" in g else (0, 0, 0, 0)
    body = tuple(float(b) for b in g["body"]) if "body" in g else (0.0, 0.0)
    return bc, body


@pytest.mark.parametrize("name", REF_FIXTURES)
def test_oracle_reproduces_reference_fixture(built, name):
    g = _load(name)
    n = int(g["n"])
    dt = float(g["dt"])
    bc, body = _ref_setup(g)
    o = Oracle(n, n, bc=bc, source=INFLOW, body=body, density=float(g["density"]))
    for f in ("q", "u", "v"):
        if f + "0" in g:
            o.set(f, g[f + "0"])
    its = [o.setup(dt, tol=1e-6, max_iter=2000)["iterations"]]
    its += [o.step(dt, 3, tol=1e-6, max_iter=2000)["iterations"] for _ in range(int(g["steps"]))]
    assert np.array_equal(its, g["iterations"])
    for f in ("q", "u", "v", "p"):
        assert np.array_equal(o.get(f), g[f]), f


@pytest.mark.gpu
@pytest.mark.parametrize("name", REF_FIXTURES)
def test_gpu_reproduces_reference_fixture(built, name):
    """The CUDA FP64 step equals the reference's own step bit for bit."""
    from cajitafluids_gb300 import Context, SolverOptions
    g = _load(name)
    n = int(g["n"])
    dt = float(g["dt"])
    bc, body = _ref_setup(g)
    c = Context(n, n)
    c.set_bc(bc)
    c.set_source(*INFLOW)
    c.set_body_force(body)
    c.set_density(float(g["density"]))
    for f in ("q", "u", "v"):
        if f + "0" in g:
            c.upload(f, g[f + "0"])
    o = SolverOptions(solver="Reference", tol=1e-6, max_iter=2000)
    its = [c.setup(dt, o)["iterations"]]
    its += [c.step(dt, 3, o)["iterations"] for _ in range(int(g["steps"]))]
    assert np.array_equal(its, g["iterations"])
    for f in ("q", "u", "v", "p"):
        assert np.array_equal(c.download(f), g[f]), f
