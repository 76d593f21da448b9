"""Mixed precision (FP32 advection and inner PCG, FP64 outer refinement)
against the FP64 oracle.

Tolerances, stated here and checked:
  * the FP64 divergence target is met on the stored (FP64) velocity field:
    ||div u||_L2 <= abs_tol (1 + 1e-9);
  * one projection from the same state: velocities within 1e-7 x max|u|
    of the FP64 result (both solved to a relative residual of 1e-11);
  * several full steps: scalar and velocity within 2e-5 x max of the FP64
    oracle (FP32 advection rounds at ~6e-8 per step).
"""
import numpy as np
import pytest

from cajitafluids_gb300.workloads import spectral_scalar, spectral_velocity
from helpers import load_state, make_pair, opts, random_state

pytestmark = pytest.mark.gpu


def _load(o, c, q, u, v):
    for f, a in (("q", q), ("u", u), ("v", v)):
        o.set(f, a)
        c.upload(f, a)


@pytest.mark.parametrize("periodic", [True, False])
def test_mixed_projection_matches_fp64(built, periodic):
    n = 96
    u, v = spectral_velocity(n, 7, periodic, kmax=12)
    rng = np.random.default_rng(1)
    # add a divergent part so the projection has work to do
    u = u + 0.05 * rng.standard_normal(u.shape)
    v = v + 0.05 * rng.standard_normal(v.shape)
    if not periodic:
        u[:, 0] = u[:, -1] = 0.0
        v[0, :] = v[-1, :] = 0.0
    q = spectral_scalar(n, 8, kmax=12)
    o, c = make_pair(n, n, periodic=(periodic, periodic), precision="mixed", quirks=1)
    _load(o, c, q, u, v)
    so = o.project(0.002, tol=1e-11, max_iter=20000)
    sg = c.project(0.002, opts(tol=1e-11, max_iter=20000))
    assert so["status"] == 0 and sg["status"] == 0
    assert sg["outer_iterations"] >= 2
    # the FP64 residual target is met on the FP64 field
    assert sg["r_norm"] <= 1e-11 * sg["b_norm"] * (1 + 1e-9)
    umax = max(np.abs(o.get("u")).max(), np.abs(o.get("v")).max())
    for f in ("u", "v"):
        d = np.abs(o.get(f) - c.download(f)).max()
        assert d <= 1e-7 * umax, (f, d, umax)


def test_mixed_abs_tol_meets_divergence_target(built):
    n = 128
    u, v = spectral_velocity(n, 3, True, kmax=16)
    rng = np.random.default_rng(2)
    u = u + 0.1 * rng.standard_normal(u.shape)
    o, c = make_pair(n, n, periodic=(True, True), precision="mixed")
    _load(o, c, spectral_scalar(n, 4, kmax=16), u, v)
    sg = c.project(0.002, opts(tol=0.0, abs_tol=1e-8, max_iter=50000))
    assert sg["status"] == 0
    assert sg["div_l2"] <= 1e-8 * (1 + 1e-9)
    l2, linf = c.div_norms()
    assert l2 == sg["div_l2"] and l2 <= 1e-8 * (1 + 1e-9)


@pytest.mark.parametrize("order", [1, 3])
def test_mixed_steps_periodic_spectral(built, order):
    n = 128
    u, v = spectral_velocity(n, 11, True, kmax=16)
    q = spectral_scalar(n, 12, kmax=16)
    dt = 0.5 / n / max(np.abs(u).max(), np.abs(v).max())
    o, c = make_pair(n, n, periodic=(True, True), precision="mixed")
    _load(o, c, q, u, v)
    for k in range(8):
        so = o.step(dt, order, tol=0.0, abs_tol=1e-8, max_iter=50000)
        sg = c.step(dt, order, opts(tol=0.0, abs_tol=1e-8, max_iter=50000))
        assert sg["status"] == 0 and sg["div_l2"] <= 1e-8 * (1 + 1e-9), (k, sg)
    qa, qb = o.get("q"), c.download("q")
    assert np.abs(qa - qb).max() <= 2e-5, np.abs(qa - qb).max()
    umax = np.abs(o.get("u")).max()
    for f in ("u", "v"):
        assert np.abs(o.get(f) - c.download(f)).max() <= 2e-5 * umax


def test_mixed_steps_walls_inflow(built):
    n = 64
    inflow = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)
    o, c = make_pair(n, n, source=inflow, precision="mixed")
    dt = 0.5 / n / 3.0
    o.setup(dt, tol=1e-10, max_iter=20000)
    c.setup(dt, opts(tol=1e-10, max_iter=20000))
    for k in range(10):
        o.step(dt, 3, tol=1e-10, max_iter=20000)
        sg = c.step(dt, 3, opts(tol=1e-10, max_iter=20000))
        assert sg["status"] == 0
    assert np.abs(o.get("q") - c.download("q")).max() <= 2e-5
    vmax = np.abs(o.get("v")).max()
    assert np.abs(o.get("v") - c.download("v")).max() <= 2e-5 * vmax


@pytest.mark.parametrize("periodic,bc", [((True, True), (0, 0, 0, 0)), ((False, False), (0, 1, 0, 0)),
                                         ((True, False), (0, 0, 0, 1))])
def test_mixed_fp32_velocity_copies(built, periodic, bc):
    """The gradient subtraction leaves the FP32 velocity copies for the next
    FP32 advection; steps that use them equal steps whose copies are made
    from the FP64 velocities (an upload in between invalidates them) bit for
    bit, on periodic, walled and mixed grids, for several steps."""
    n = 96
    inflow = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)
    pairs = [make_pair(n, n, periodic=periodic, bc=bc, source=inflow, precision="mixed", precon_mg=True)
             for _ in range(2)]
    rng = np.random.default_rng(11)
    st = random_state(pairs[0][0], rng)
    for o, c in pairs:
        load_state(o, c, st)
    dt = 0.5 / n / 3.0
    so = opts(tol=1e-9, max_iter=500, precon="PFMG")
    ca, cb = pairs[0][1], pairs[1][1]
    for k in range(4):
        sa = ca.step(dt, 3, so)
        sb = cb.step(dt, 3, so)
        cb.upload("u", cb.download("u"))  # FP64 round trip: same values, copies invalidated
        assert sa["iterations"] == sb["iterations"], k
    for f in ("q", "u", "v", "p"):
        assert np.array_equal(ca.download(f), cb.download(f)), f
