"""Configs 0 and 1 of the benchmark plan at their full sizes, in FP64 with the
reference's own solver form (Jacobi-preconditioned CG), against the oracle.

Config 0: 256^2, walls, zero start, the inflow box (Q = 1, v = 3), linear
values, CG to a relative residual of 1e-8: setup + all 100 steps, bit for
bit (the iteration count and ||div u|| of every projection, and a SHA-256
digest of the final q, u, v, p).
Config 1: 1024^2, the same inflow, gravity (0, -9.8) scaled by the quantity,
cubic values, CG to 1e-10: setup + the first two steps bit for bit (what the
oracle affords: about a minute per projection), then the run continues to
its 500 steps on the GPU and every projection must converge.

The fixtures (tests/golden/config0_256_full.npz, config1_1024_head.npz) are
oracle runs made by tests/golden/make_golden.py --long; the oracle equals
the reference's own code bit for bit (tests/test_reference_pin.py).
"""
import hashlib
import os

import numpy as np
import pytest

from cajitafluids_gb300 import Context, SolverOptions
from cajitafluids_gb300.workloads import config0, config1

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _digest(c):
    h = hashlib.sha256()
    for f in ("q", "u", "v", "p"):
        h.update(np.ascontiguousarray(c.download(f), dtype=np.float64).tobytes())
    return h.hexdigest()


def _context(w):
    c = Context(w.nx, w.ny)
    c.set_bc(w.bc)
    c.set_source(*w.source, mode=w.source_mode)
    c.set_body_force(w.body, w.body_density_scaled)
    c.set_density(w.density)
    return c


def test_config0_full_run_bit_for_bit(built):
    g = dict(np.load(os.path.join(GOLDEN, "config0_256_full.npz")))
    w = config0(steps=int(g["steps"]))
    c = _context(w)
    o = SolverOptions(tol=w.tol, max_iter=20000, precon="Diagonal")
    st = [c.setup(w.dt, o, raise_on_maxit=True)]
    st += [c.step(w.dt, w.order, o, raise_on_maxit=True) for _ in range(w.steps)]
    assert np.array_equal([s["iterations"] for s in st], g["iterations"])
    assert np.array_equal([s["div_l2"] for s in st], g["div_l2"])
    assert np.array_equal([s["div_linf"] for s in st], g["div_linf"])
    assert _digest(c) == str(g["digest"])


def test_config1_head_bit_for_bit_then_full_run(built):
    g = dict(np.load(os.path.join(GOLDEN, "config1_1024_head.npz")))
    w = config1(steps=500)
    c = _context(w)
    o = SolverOptions(tol=w.tol, max_iter=50000, precon="Diagonal")
    st = [c.setup(w.dt, o, raise_on_maxit=True)]
    st += [c.step(w.dt, w.order, o, raise_on_maxit=True) for _ in range(int(g["steps"]))]
    assert np.array_equal([s["iterations"] for s in st], g["iterations"])
    assert np.array_equal([s["div_l2"] for s in st], g["div_l2"])
    assert _digest(c) == str(g["digest"])
    # the rest of the 500 steps: one device-side loop, every solve converged
    last = c.steps(w.steps - int(g["steps"]), w.dt, w.order, o, raise_on_maxit=True)
    assert last["unconverged"] == 0
    assert np.isfinite(c.download("q")).all()
