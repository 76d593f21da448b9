"""cf_steps: Solver::solve's step loop (src/Solver.hpp:149-177) enqueued on
the device with one synchronisation; the same state as the same number of
cf_step calls, bit for bit, and a count of the solves that did not
converge."""
import numpy as np
import pytest

from helpers import load_state, make_pair, opts, random_state

pytestmark = pytest.mark.gpu

INFLOW = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("precon", ["PFMG", "Diagonal"])
@pytest.mark.parametrize("periodic", [False, True])
def test_steps_match_single_steps(built, precision, precon, periodic):
    n = 64
    per = (periodic, periodic)
    src = None if periodic else INFLOW
    pairs = [make_pair(n, n, periodic=per, source=src, precision=precision, precon_mg=precon == "PFMG")
             for _ in range(2)]
    st = random_state(pairs[0][0], np.random.default_rng(5), smooth=True)
    for o, c in pairs:
        load_state(o, c, st)
    dt = 0.5 / n / 3.0
    so = opts(tol=1e-9, max_iter=3000, precon=precon)
    ca, cb = pairs[0][1], pairs[1][1]
    for _ in range(5):
        sa = ca.step(dt, 3, so)
    sb = cb.steps(5, dt, 3, so)
    assert sb["unconverged"] == 0
    assert sa["iterations"] == sb["iterations"] and sa["div_l2"] == sb["div_l2"]
    for f in ("q", "u", "v", "p"):
        assert np.array_equal(ca.download(f), cb.download(f)), f


def test_steps_count_unconverged(built):
    from cajitafluids_gb300 import CfError
    from cajitafluids_gb300 import _lib as L
    n = 48
    o, c = make_pair(n, n, source=INFLOW, precon_mg=True)
    load_state(o, c, random_state(o, np.random.default_rng(3)))
    dt = 0.5 / n / 3.0
    s = c.steps(3, dt, 3, opts(tol=1e-14, max_iter=1, precon="PFMG"))
    assert s["unconverged"] == 3 and s["status"] == 1
    with pytest.raises(CfError) as e:
        c.steps(2, dt, 3, opts(tol=1e-14, max_iter=1, precon="PFMG"), raise_on_maxit=True)
    assert e.value.code == L.CF_ERR_NOT_CONVERGED
    s = c.steps(0, dt, 3, opts(precon="PFMG"))
    assert s["unconverged"] == 0
    s = c.steps(2, dt, 3, opts(tol=1e-9, max_iter=500, precon="PFMG"))
    assert s["unconverged"] == 0 and s["status"] == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_graphs_follow_changes(built, precision):
    """cf_steps runs each step as one cached graph (ghost fill, advection,
    inputs, projection); a change of dt, value order, body force or inflow
    between calls must rebuild it: the same states as cf_step calls with the
    same changes."""
    n = 64
    pairs = [make_pair(n, n, source=INFLOW, precision=precision, precon_mg=True) for _ in range(2)]
    st = random_state(pairs[0][0], np.random.default_rng(9), smooth=True)
    for o, c in pairs:
        load_state(o, c, st)
    so = opts(tol=1e-9, max_iter=3000, precon="PFMG")
    ca, cb = pairs[0][1], pairs[1][1]
    dt = 0.5 / n / 3.0
    plan = [(2, dt, 3, None), (2, 0.7 * dt, 3, None), (1, 0.7 * dt, 1, None), (2, 0.7 * dt, 3, (0.0, -9.8)),
            (2, 0.7 * dt, 3, ((0.40, 0.10), (0.20, 0.10), (0.0, 2.0), 0.5))]
    for k, d, order, change in plan:
        for c in (ca, cb):
            if change is not None and len(change) == 2:
                c.set_body_force(change, density_scaled=True)
            elif change is not None:
                c.set_source(*change)
        for _ in range(k):
            ca.step(d, order, so)
        cb.steps(k, d, order, so)
        for f in ("q", "u", "v"):
            assert np.array_equal(ca.download(f), cb.download(f)), (k, d, order, change, f)
