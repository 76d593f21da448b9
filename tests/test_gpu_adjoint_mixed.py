"""Mixed-precision adjoint (cf_forward_checkpointed / cf_backward on a mixed
context): FP32 reverse advection (k_adj_advect32), transposed projection
with the mixed PCG on pair arrays, checkpoints of the mixed state.

Checks:
  * dot-product test on the scalar transport (q(T) is linear in q(0) while
    the velocity evolves on its own): <q_T(dq), y> = <dq, J^T y> to FP32
    round-off, cubic and linear values, walls and periodic;
  * the gradient agrees with the FP64 adjoint of the same problem (FP32 bulk:
    1e-4 relative in the 2-norm per field, and for dL/d(rate)), and its
    directional derivatives with central differences of the FP64 forward;
  * gradients are bit-for-bit reproducible and independent of the
    checkpoint spacing (the recomputation repeats the mixed forward exactly
    and the reverse advection has no atomics);
  * the reference's default inputs (clamp-form source with an inflow
    velocity, density-scaled buoyancy) agree with the FP64 adjoint;
  * a trace that moves a full cell fails the call with CF_ERR_UNSUPPORTED.
"""
import numpy as np
import pytest

from cajitafluids_gb300 import CfError, Context, SolverOptions
from cajitafluids_gb300 import _lib as L
from cajitafluids_gb300.workloads import gaussian_blobs, spectral_velocity

pytestmark = pytest.mark.gpu

N = 48
STEPS = 8
PRECONS = ("Diagonal", "PFMG")


def opts_for(precon, mixed=True):
    # the mixed solves stop well above the double-float floor; the FP64
    # reference runs to 1e-13
    return SolverOptions(tol=1e-10 if mixed else 1e-13, max_iter=20000, precon=precon)


def make_ctx(mixed, rate=0.0, periodic=False):
    c = Context(N, N, periodic=(periodic, periodic), precision="mixed" if mixed else "fp64")
    c.set_density(0.1)
    c.set_quirks(L.CF_FIX_Q1)
    if rate:
        c.set_source((0.45, 0.10), (0.10, 0.05), (0.0, 0.0), rate, mode=1)
    return c


def initial(periodic=False, seed=3):
    u, v = spectral_velocity(N, seed, periodic, kmax=6)
    q = gaussian_blobs(N, seed + 1, count=4, sigma=0.08)
    return q, 0.6 * u, 0.6 * v


def dt_for(u, v):
    return 0.4 / N / max(np.abs(u).max(), np.abs(v).max())


def run(c, q, u, v, dt, every=3, opts=None, order=3):
    c.upload("q", q)
    c.upload("u", u)
    c.upload("v", v)
    c.forward_checkpointed(STEPS, every, dt, order, opts or opts_for("Diagonal"))
    return c.download("q"), c.download("u"), c.download("v")


@pytest.mark.parametrize("order", [3, 1])
@pytest.mark.parametrize("periodic", [False, True])
def test_mixed_dot_product_scalar_transport(periodic, order):
    q, u, v = initial(periodic)
    dt = dt_for(u, v)
    c = make_ctx(True, periodic=periodic)
    rng = np.random.default_rng(0)
    dq = rng.standard_normal(q.shape)
    y = rng.standard_normal(q.shape)
    q1, _, _ = run(c, dq, u, v, dt, order=order)
    g = c.backward(y)
    lhs = float(np.sum(q1 * y))
    rhs = float(np.sum(dq * g["q"]))
    assert abs(lhs - rhs) <= 1e-5 * float(np.sum(np.abs(q1 * y))), (lhs, rhs)


@pytest.mark.parametrize("precon", PRECONS)
@pytest.mark.parametrize("periodic", [False, True])
def test_mixed_gradient_matches_fp64_adjoint(periodic, precon):
    q0, u0, v0 = initial(periodic)
    dt = dt_for(u0, v0)
    rate = 0.0 if periodic else 2.0
    target = gaussian_blobs(N, 11, count=4, sigma=0.08)
    rng = np.random.default_rng(5)
    grads, ctxs = {}, {}
    for mixed in (False, True):
        c = make_ctx(mixed, rate, periodic)
        cu = np.random.default_rng(6).standard_normal(c.owned_shape("u")) * 0.1
        cv = np.random.default_rng(7).standard_normal(c.owned_shape("v")) * 0.1
        qT, _, _ = run(c, q0, u0, v0, dt, opts=opts_for(precon, mixed))
        grads[mixed] = c.backward(qT - target, cu, cv)
        ctxs[mixed] = (c, cu, cv)
    g64, g32 = grads[False], grads[True]
    for f in ("q", "u", "v"):
        rel = np.linalg.norm(g32[f] - g64[f]) / np.linalg.norm(g64[f])
        assert rel <= 1e-4, (f, rel)
    if not periodic:
        assert abs(g32["rate"] - g64["rate"]) <= 1e-4 * abs(g64["rate"]), (g32["rate"], g64["rate"])
    # directional derivative against central differences of the FP64 forward
    c, cu, cv = ctxs[False]

    def loss(q, u, v):
        qT, uT, vT = run(c, q, u, v, dt, opts=opts_for(precon, False))
        return 0.5 * float(np.sum((qT - target) ** 2)) + float(np.sum(cu * uT)) + float(np.sum(cv * vT))

    dq = rng.standard_normal(q0.shape)
    du = rng.standard_normal(u0.shape)
    dv = rng.standard_normal(v0.shape)
    if not periodic:
        du[:, 0] = du[:, -1] = 0.0
        dv[0, :] = dv[-1, :] = 0.0
    h = 1e-5
    fd = (loss(q0 + h * dq, u0 + h * du, v0 + h * dv) - loss(q0 - h * dq, u0 - h * du, v0 - h * dv)) / (2 * h)
    ad = float(np.sum(g32["q"] * dq) + np.sum(g32["u"] * du) + np.sum(g32["v"] * dv))
    assert abs(fd - ad) <= 1e-4 * abs(fd), (fd, ad)


@pytest.mark.parametrize("buoyancy", [False, True])
def test_mixed_default_physics_matches_fp64_adjoint(buoyancy):
    """The reference's default inputs (clamp-form source with an inflow
    velocity, density-scaled buoyancy) in the mixed adjoint against the FP64
    adjoint of the same problem."""
    q0, u0, v0 = initial()
    dt = 0.4 / N / max(np.abs(u0).max(), np.abs(v0).max(), 3.0)
    target = gaussian_blobs(N, 11, count=4, sigma=0.08)
    grads = {}
    for mixed in (False, True):
        c = Context(N, N, precision="mixed" if mixed else "fp64")
        c.set_density(0.1)
        c.set_quirks(L.CF_FIX_Q1)
        c.set_source((0.40, 0.10), (0.20, 0.10), (0.0, 3.0), 0.8, mode=0)
        if buoyancy:
            c.set_body_force((0.0, -9.8), density_scaled=True)
        qT, _, _ = run(c, q0, u0, v0, dt, opts=opts_for("PFMG", mixed))
        grads[mixed] = c.backward(qT - target)
    g64, g32 = grads[False], grads[True]
    for f in ("q", "u", "v"):
        rel = np.linalg.norm(g32[f] - g64[f]) / np.linalg.norm(g64[f])
        assert rel <= 1e-4, (f, rel)
    assert g64["rate"] != 0.0
    assert abs(g32["rate"] - g64["rate"]) <= 1e-4 * abs(g64["rate"]), (g32["rate"], g64["rate"])


def test_mixed_gradient_is_reproducible_and_schedule_independent():
    q0, u0, v0 = initial()
    dt = dt_for(u0, v0)
    c = make_ctx(True, 1.0)
    y = np.random.default_rng(2).standard_normal(q0.shape)
    grads = []
    for every in (3, 3, 1, 8):
        run(c, q0, u0, v0, dt, every, opts=opts_for("PFMG"))
        grads.append(c.backward(y))
    for g in grads[1:]:
        for f in ("q", "u", "v"):
            assert np.array_equal(g[f], grads[0][f]), f
        assert g["rate"] == grads[0]["rate"]


def test_mixed_trace_too_long_is_rejected():
    q0, u0, v0 = initial()
    c = make_ctx(True)
    run(c, q0, u0, v0, 3.0 * dt_for(u0, v0) * 2.5)   # traces move more than one cell
    with pytest.raises(CfError) as e:
        c.backward(q0)
    assert e.value.code == L.CF_ERR_UNSUPPORTED
