"""Hand-written adjoint of the step (cf_forward_checkpointed / cf_backward).

Checks:
  * dot-product test: the velocity evolves independently of the scalar, so
    q(T) is linear in q(0) and <q_T(dq), y> must equal <dq, J^T y> to
    round-off (the transpose of the interpolation scatter);
  * central finite differences of the FP64 forward on seeded directions in
    q(0), u(0), v(0) and the inflow rate, with the Jacobi ("Diagonal") and
    the multigrid ("PFMG") preconditioner, for a loss that mixes the scalar
    misfit 1/2 |q(T) - target|^2 with linear terms in u(T), v(T);
    tolerance 1e-5 relative to the directional derivative (the CG solves run
    to a relative residual of 1e-13 so the forward is smooth to far below
    the FD step);
  * gradients are bit-for-bit reproducible and do not depend on the
    checkpoint spacing;
  * the reference's default inputs (clamp-form source with an inflow
    velocity, density-scaled buoyancy) against central differences too, with
    dL/dQ for the clamp level;
  * unsupported settings (the Q1 quirk's projection, warm starts) return
    CF_ERR_UNSUPPORTED, a backward without a forward CF_ERR_INVALID.
A torch.autograd.Function over the same contract is exercised at the end.
"""
import numpy as np
import pytest

from cajitafluids_gb300 import CfError, Context, SolverOptions
from cajitafluids_gb300 import _lib as L
from cajitafluids_gb300.workloads import gaussian_blobs, spectral_velocity

pytestmark = pytest.mark.gpu

N = 48
STEPS = 8
OPTS = SolverOptions(tol=1e-13, max_iter=20000)
PRECONS = ("Diagonal", "PFMG")


def opts_for(precon):
    return SolverOptions(tol=1e-13, max_iter=20000, precon=precon)


def make_ctx(rate=0.0, periodic=False):
    c = Context(N, N, periodic=(periodic, periodic))
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


def run(c, q, u, v, dt, every=3, opts=OPTS):
    c.upload("q", q)
    c.upload("u", u)
    c.upload("v", v)
    c.forward_checkpointed(STEPS, every, dt, 3, opts)
    return c.download("q"), c.download("u"), c.download("v")


@pytest.mark.parametrize("precon", PRECONS)
def test_dot_product_test_scalar_transport(precon):
    q, u, v = initial()
    dt = dt_for(u, v)
    c = make_ctx()
    rng = np.random.default_rng(0)
    dq = rng.standard_normal(q.shape)
    y = rng.standard_normal(q.shape)
    q1, _, _ = run(c, dq, u, v, dt, opts=opts_for(precon))
    g = c.backward(y)
    lhs = float(np.sum(q1 * y))
    rhs = float(np.sum(dq * g["q"]))
    assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + np.sum(np.abs(q1 * y)))


@pytest.mark.parametrize("precon", PRECONS)
@pytest.mark.parametrize("periodic", [False, True])
def test_gradient_matches_central_differences(periodic, precon):
    q0, u0, v0 = initial(periodic)
    dt = dt_for(u0, v0)
    rate = 0.0 if periodic else 2.0
    c = make_ctx(rate, periodic)
    target = gaussian_blobs(N, 11, count=4, sigma=0.08)
    rng = np.random.default_rng(5)
    cu = rng.standard_normal(c.owned_shape("u")) * 0.1
    cv = rng.standard_normal(c.owned_shape("v")) * 0.1

    def loss(q, u, v, r=rate):
        if not periodic:
            c.set_source((0.45, 0.10), (0.10, 0.05), (0.0, 0.0), r, mode=1)
        qT, uT, vT = run(c, q, u, v, dt, opts=opts_for(precon))
        return 0.5 * float(np.sum((qT - target) ** 2)) + float(np.sum(cu * uT)) + float(np.sum(cv * vT)), qT

    L0, qT = loss(q0, u0, v0)
    g = c.backward(qT - target, cu, cv)
    h = 1e-5
    for k in range(4):
        dq = rng.standard_normal(q0.shape) * (k in (0, 3))
        du = rng.standard_normal(u0.shape) * (k in (1, 3))
        dv = rng.standard_normal(v0.shape) * (k in (2, 3))
        if not periodic:
            du[:, 0] = du[:, -1] = 0.0
            dv[0, :] = dv[-1, :] = 0.0
        lp, _ = loss(q0 + h * dq, u0 + h * du, v0 + h * dv)
        lm, _ = loss(q0 - h * dq, u0 - h * du, v0 - h * dv)
        fd = (lp - lm) / (2 * h)
        ad = float(np.sum(g["q"] * dq) + np.sum(g["u"] * du) + np.sum(g["v"] * dv))
        assert abs(fd - ad) <= 1e-5 * abs(ad) + 1e-9, (k, fd, ad)
    if not periodic:
        hr = 1e-5
        lp, _ = loss(q0, u0, v0, rate + hr)
        lm, _ = loss(q0, u0, v0, rate - hr)
        fd = (lp - lm) / (2 * hr)
        assert abs(fd - g["rate"]) <= 1e-5 * abs(g["rate"]), (fd, g["rate"])


def default_physics_ctx(Q=0.8, mixed=False, buoyancy=True):
    """The reference's default inputs (examples/advection.cpp): a clamp-form
    quantity source q = max(q, Q) with an inflow velocity (0, 3) in the box,
    and (config 1) buoyancy scaled by the density."""
    c = Context(N, N, precision="mixed" if mixed else "fp64")
    c.set_density(0.1)
    c.set_quirks(L.CF_FIX_Q1)
    c.set_source((0.40, 0.10), (0.20, 0.10), (0.0, 3.0), Q, mode=0)
    if buoyancy:
        c.set_body_force((0.0, -9.8), density_scaled=True)
    return c


def default_physics_dt(u, v):
    return 0.4 / N / max(np.abs(u).max(), np.abs(v).max(), 3.0)


@pytest.mark.parametrize("precon", PRECONS)
@pytest.mark.parametrize("buoyancy", [False, True])
def test_gradient_of_default_physics_matches_central_differences(precon, buoyancy):
    """Clamp-form source with a velocity inflow, with and without the
    density-scaled buoyancy: directional derivatives in q, u, v and dL/dQ
    (the clamp level) against central differences of the FP64 forward."""
    q0, u0, v0 = initial()
    dt = default_physics_dt(u0, v0)
    Q = 0.8
    c = default_physics_ctx(Q, buoyancy=buoyancy)
    target = gaussian_blobs(N, 11, count=4, sigma=0.08)
    rng = np.random.default_rng(7)
    cu = rng.standard_normal(c.owned_shape("u")) * 0.1
    cv = rng.standard_normal(c.owned_shape("v")) * 0.1

    def loss(q, u, v, level=Q):
        c.set_source((0.40, 0.10), (0.20, 0.10), (0.0, 3.0), level, mode=0)
        qT, uT, vT = run(c, q, u, v, dt, opts=opts_for(precon))
        return 0.5 * float(np.sum((qT - target) ** 2)) + float(np.sum(cu * uT)) + float(np.sum(cv * vT)), qT

    _, qT = loss(q0, u0, v0)
    g = c.backward(qT - target, cu, cv)
    h = 1e-5
    for k in range(3):
        dq = rng.standard_normal(q0.shape) * (k in (0, 2))
        du = rng.standard_normal(u0.shape) * (k in (1, 2))
        dv = rng.standard_normal(v0.shape) * (k in (1, 2))
        du[:, 0] = du[:, -1] = 0.0
        dv[0, :] = dv[-1, :] = 0.0
        lp, _ = loss(q0 + h * dq, u0 + h * du, v0 + h * dv)
        lm, _ = loss(q0 - h * dq, u0 - h * du, v0 - h * dv)
        fd = (lp - lm) / (2 * h)
        ad = float(np.sum(g["q"] * dq) + np.sum(g["u"] * du) + np.sum(g["v"] * dv))
        assert abs(fd - ad) <= 1e-5 * abs(ad) + 1e-9, (k, fd, ad)
    lp, _ = loss(q0, u0, v0, Q + h)
    lm, _ = loss(q0, u0, v0, Q - h)
    fd = (lp - lm) / (2 * h)
    assert g["rate"] != 0.0
    assert abs(fd - g["rate"]) <= 1e-5 * abs(g["rate"]), (fd, g["rate"])


def test_gradient_is_reproducible_and_schedule_independent():
    q0, u0, v0 = initial()
    dt = dt_for(u0, v0)
    c = make_ctx(1.0)
    y = np.random.default_rng(2).standard_normal(q0.shape)
    grads = []
    for every in (3, 3, 1, 8):
        run(c, q0, u0, v0, dt, every)
        grads.append(c.backward(y))
    for g in grads[1:]:
        for f in ("q", "u", "v"):
            assert np.array_equal(g[f], grads[0][f]), f
        assert g["rate"] == grads[0]["rate"]


def test_unsupported_and_invalid_settings():
    q0, u0, v0 = initial()
    dt = dt_for(u0, v0)
    c = Context(N, N)
    c.set_quirks(0)                      # Q1 quirk active with SOLID y-walls
    run(c, q0, u0, v0, dt)
    with pytest.raises(CfError) as e:
        c.backward(q0)
    assert e.value.code == L.CF_ERR_UNSUPPORTED
    c2 = Context(N, N)
    with pytest.raises(CfError) as e:
        c2.backward(q0)
    assert e.value.code == L.CF_ERR_INVALID
    c3 = Context(N, N)
    c3.set_warm_start(True)
    with pytest.raises(CfError) as e:
        c3.forward_checkpointed(2, 1, dt)
    assert e.value.code == L.CF_ERR_UNSUPPORTED
    c4 = make_ctx()
    run(c4, q0, u0, v0, 3.0 * dt_for(u0, v0) * 2.5)   # traces move more than one cell
    with pytest.raises(CfError) as e:
        c4.backward(q0)
    assert e.value.code == L.CF_ERR_UNSUPPORTED


def test_torch_autograd_function_contract():
    torch = pytest.importorskip("torch")
    q0, u0, v0 = initial()
    dt = dt_for(u0, v0)
    c = make_ctx()
    target = torch.tensor(gaussian_blobs(N, 11, count=4, sigma=0.08))

    class Steps(torch.autograd.Function):
        @staticmethod
        def forward(ctx, q, u, v):
            qT, _, _ = run(c, q.detach().numpy(), u.detach().numpy(), v.detach().numpy(), dt)
            return torch.tensor(qT)

        @staticmethod
        def backward(ctx, gq):
            g = c.backward(gq.detach().numpy())
            return torch.tensor(g["q"]), torch.tensor(g["u"]), torch.tensor(g["v"])

    q = torch.tensor(q0, requires_grad=True)
    u = torch.tensor(u0, requires_grad=True)
    v = torch.tensor(v0, requires_grad=True)
    loss = 0.5 * ((Steps.apply(q, u, v) - target) ** 2).sum()
    loss.backward()
    qT, _, _ = run(c, q0, u0, v0, dt)
    g = c.backward(qT - target.numpy())
    assert np.array_equal(q.grad.numpy(), g["q"]) and np.array_equal(u.grad.numpy(), g["u"])
