"""The oracle against the reference's own code (CPU, no GPU).

oracle/_ref/libcfref.so is the reference's src/*.hpp compiled unchanged
against serial Kokkos/Cajita/MPI stand-ins (oracle/refshim), run through
createSolver("serial", ...) with the "Reference" solver
(src/Solver.hpp:283-350, src/VelocityCorrector.hpp:297-323).  The reference
hard-codes the solver's tolerance and iteration limit (1e-6, 2000,
src/VelocityCorrector.hpp:103-104) and cubic values (src/TimeIntegrator.hpp:
112-113), so the oracle runs with those.

Whole steps, bit for bit: q, u, v, the pressure and every solve's iteration
count, over walls of both kinds, body forces, rectangular and offset
domains.  Then the reference's functors entity by entity against the
oracle's inputs and matrix.  The GPU side is pinned to the oracle bit for bit
by the -m gpu tests, and to fixtures written from this reference run by
tests/golden/make_golden.py (tests/test_golden.py).

Skipped where the reference's sources are not on the machine.
"""
import numpy as np
import pytest

from oracle import Oracle
from oracle import reference as R

pytestmark = pytest.mark.skipif(not R.available(), reason="the reference's sources are not on this machine")

INFLOW = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)


def _run_both(nx, ny, steps, lo=(0.0, 0.0), hi=None, bc=(0, 0, 0, 0), source=INFLOW, body=(0.0, 0.0), density=0.1,
              dt=None, state=None):
    if hi is None:
        hi = (lo[0] + 1.0, lo[1] + ny / nx)
    dx = (hi[0] - lo[0]) / nx
    if dt is None:
        dt = 0.5 * dx / 3.0
    prm = R.params(nx, ny, lo=lo, hi=hi, bc=bc, source=source, body=body, density=density, dt=dt)
    state = state or {}
    ref = R.run(prm, state.get("q"), state.get("u"), state.get("v"), steps=steps)
    o = Oracle(nx, ny, lo=lo, hi=hi, bc=bc, source=source, body=body, density=density)
    for f in ("q", "u", "v"):
        if f in state:
            o.set(f, state[f])
    its = [o.setup(dt, tol=1e-6, max_iter=2000)["iterations"]]
    for _ in range(steps):
        its.append(o.step(dt, 3, tol=1e-6, max_iter=2000)["iterations"])
    return ref, o, its


def _assert_same(ref, o, its):
    assert list(ref["iterations"]) == its
    assert not ref["status"].any()
    for f in ("q", "u", "v", "p"):
        a, b = ref[f], o.get(f)
        assert np.array_equal(a, b), (f, np.count_nonzero(a != b), float(np.abs(a - b).max()))


@pytest.mark.parametrize("n,steps,bc,body", [
    (32, 4, (0, 0, 0, 0), (0.0, 0.0)),         # config 0's problem: walls, inflow, zero start
    (48, 4, (0, 1, 0, 1), (0.0, -9.8)),        # FREE bottom and top, gravity
    (64, 3, (1, 0, 0, 0), (0.3, -9.8)),        # FREE left wall, oblique force
    (40, 3, (1, 1, 1, 1), (0.0, -1.0)),        # all FREE
])
def test_reference_steps_bit_for_bit(built, n, steps, bc, body):
    ref, o, its = _run_both(n, n, steps, bc=bc, body=body)
    _assert_same(ref, o, its)


def test_reference_rectangular_offset_domain(built):
    """A 48 x 32 grid on [0.25, 1.75] x [-0.5, 0.5] (square cells, a low
    corner off the origin) and an inflow box that straddles cell centres."""
    src = ((0.6, -0.35), (0.2, 0.1), (0.5, 2.0), 0.7)
    ref, o, its = _run_both(48, 32, 3, lo=(0.25, -0.5), hi=(1.75, 0.5), source=src, body=(0.2, -3.0))
    _assert_same(ref, o, its)


def test_reference_from_a_random_state(built):
    """Seeded random quantity and velocities (walls zeroed by the first
    _addInputs), so every spline tap and every matrix row is exercised."""
    n = 40
    rng = np.random.default_rng(11)
    state = {"q": rng.uniform(0.0, 1.0, (n, n)), "u": rng.standard_normal((n, n + 1)) * 0.3,
             "v": rng.standard_normal((n + 1, n)) * 0.3}
    ref, o, its = _run_both(n, n, 3, bc=(0, 1, 0, 0), body=(0.0, -2.0), dt=0.25 / n, state=state)
    _assert_same(ref, o, its)


def test_reference_solve_loop_writes_and_steps(built):
    """Solver::solve(t_final, write_freq) (src/Solver.hpp:149-177): setup,
    then steps while time < t_final, a write before the loop and every
    write_freq steps; the final fields equal setup + the same number of
    oracle steps."""
    n = 24
    dt = 0.5 / n / 3.0
    prm = R.params(n, n, source=INFLOW, density=0.1, dt=dt)
    ref = R.run(prm, t_final=7.5 * dt, write_freq=3)
    steps = len(ref["iterations"]) - 1
    assert steps == 8   # 8 steps take the time from 0 past 7.5 dt
    assert ref["writes"] == 1 + 3   # before the loop, and after steps 0, 3, 6
    o = Oracle(n, n, source=INFLOW, density=0.1)
    its = [o.setup(dt, tol=1e-6, max_iter=2000)["iterations"]]
    its += [o.step(dt, 3, tol=1e-6, max_iter=2000)["iterations"] for _ in range(steps)]
    _assert_same(ref, o, its)


def test_reference_functors_match_oracle_inputs(built):
    """InflowSource<2>, BodyForce<2> and BoundaryCondition<2> applied by the
    reference's own functors to every owned entity in the order _addInputs
    uses (src/Solver.hpp:181-263) equal the oracle's inputs, bit for bit."""
    n = 20
    dx = 1.0 / n
    dt = 0.37 * dx
    src = ((0.3, 0.2), (0.35, 0.3), (-0.8, 1.7), 0.6)
    body = (0.4, -9.8)
    bc = (0, 1, 0, 0)
    prm = R.params(n, n, bc=bc, source=src, body=body, dt=dt)
    rng = np.random.default_rng(4)
    q = rng.uniform(0.0, 1.0, (n, n))
    u = rng.standard_normal((n, n + 1))
    v = rng.standard_normal((n + 1, n))
    o = Oracle(n, n, bc=bc, source=src, body=body)
    for f, a in (("q", q), ("u", u), ("v", v)):
        o.set(f, a)
    o.add_inputs(dt)
    low = -3.0 * dx
    qe, ue, ve = q.copy(), u.copy(), v.copy()
    for gj in range(n):
        for gi in range(n):
            x = low + ((gi + 3) + 0.5) * dx
            y = low + ((gj + 3) + 0.5) * dx
            qe[gj, gi] = R.functor(prm, "cell_inflow", gi, gj, x, y, qe[gj, gi])
    for gj in range(n):
        for gi in range(n + 1):
            x = low + (gi + 3) * dx
            y = low + ((gj + 3) + 0.5) * dx
            w = R.functor(prm, "iface_inflow", gi, gj, x, y, ue[gj, gi])
            w = R.functor(prm, "iface_body", gi, gj, x, y, w)
            ue[gj, gi] = R.functor(prm, "iface_bc", gi, gj, x, y, w)
    for gj in range(n + 1):
        for gi in range(n):
            x = low + ((gi + 3) + 0.5) * dx
            y = low + (gj + 3) * dx
            w = R.functor(prm, "jface_inflow", gi, gj, x, y, ve[gj, gi])
            w = R.functor(prm, "jface_body", gi, gj, x, y, w)
            ve[gj, gi] = R.functor(prm, "jface_bc", gi, gj, x, y, w)
    assert np.array_equal(o.get("q"), qe)
    assert np.array_equal(o.get("u"), ue)
    assert np.array_equal(o.get("v"), ve)


@pytest.mark.parametrize("bc", [(0, 0, 0, 0), (1, 0, 1, 0), (0, 1, 1, 0)])
def test_reference_build_matrix_matches_oracle_operator(built, bc):
    """The reference's matrix (initializeMatrixValues + build_matrix,
    src/VelocityCorrector.hpp:116-144, src/BoundaryConditions.hpp:57-97)
    entry for entry against the oracle's operator: nine matrix-vector
    products with the indicator of cells (i, j) = (a, b) mod 3 give every
    diagonal entry and every neighbour leg."""
    nx, ny = 13, 11
    dt, density = 0.003, 0.7
    hi = (1.0, ny / nx)
    dx = 1.0 / nx
    scale = dt / ((density * dx) * dx)
    prm = R.params(nx, ny, hi=hi, bc=bc, density=density, dt=dt)
    o = Oracle(nx, ny, hi=hi, bc=bc, density=density)
    legs = ((-1, 0), (1, 0), (0, -1), (0, 1))   # stencil entries 1..4: W, E, S, N
    for a in range(3):
        for b in range(3):
            p = np.zeros((ny, nx))
            p[b::3, a::3] = 1.0
            ap = o.matvec(dt, p)
            for gj in range(b, ny, 3):
                for gi in range(a, nx, 3):
                    m = R.functor(prm, "build_matrix", gi, gj, scale=scale)
                    assert ap[gj, gi] == m[0], (gi, gj)
                    for e, (di, dj) in enumerate(legs, start=1):
                        ni, nj = gi - di, gj - dj   # the cell whose leg e points at (gi, gj)
                        if 0 <= ni < nx and 0 <= nj < ny:
                            mn = R.functor(prm, "build_matrix", ni, nj, scale=scale)
                            assert ap[nj, ni] == mn[e], (ni, nj, e)
