"""CPU checks of the oracle (no GPU).

Pins, in the order of the reference's own tests and then the known answers
the hot path must satisfy:
  * Mesh / ProblemManager conventions of tests/tstMesh.cpp:16-69 and
    tests/tstProblemManager.cpp:23-98 (cell size, domain indices, ghosted
    extents, halo encoding across a periodic seam);
  * interpolation reproduces constants and affine fields; the cubic B-spline
    at a grid point is the (1, 4, 1)/6 stencil;
  * rk3 under a uniform velocity traces x0 - dt U;
  * the discrete divergence of a streamfunction MAC field vanishes;
  * the 5-point matrix equals BoundaryCondition::build_matrix entry for
    entry and is symmetric; CG matches a sparse direct solve;
  * the fixed-order dot product agrees with numpy's;
  * the inputs (inflow box at entity positions, body force, SOLID walls), the
    rk3 trace with and without quirk Q3, the divergence of an affine field and
    the gradient subtraction with quirk Q1.
"""
import numpy as np
import pytest

import oracle
from cajitafluids_gb300.workloads import mac_from_streamfunction
from oracle import Oracle


# ---- reference tests: tests/tstMesh.cpp, tests/tstProblemManager.cpp ----
def test_mesh_basic_parameters():
    """MeshTest.BasicParameters: 512 cells on a unit box."""
    o = Oracle(512, 512)
    # cellSize == boxWidth / boxCells; exercised through a sample of u = x
    ny, nx = o.shape("u")
    assert (ny, nx) == (512, 513)
    x = np.arange(nx) / 512.0
    o.set("u", np.tile(x, (ny, 1)))
    o.fill_ghosts()
    xy = np.array([[0.25, 0.5], [0.5, 0.5]])
    assert np.allclose(o.sample("u", 1, xy), [0.25, 0.5], atol=1e-14)


def test_mesh_local_grid_extents():
    """MeshTest.LocalGridSetup: ghosted I-face extent is N + 2*3 + 1 by N + 2*3."""
    n = 64
    o = Oracle(n, n)
    g = o.get_ghosted("u")
    assert g.shape == (n + 2 * 3, n + 2 * 3 + 1)
    assert o.get_ghosted("v").shape == (n + 2 * 3 + 1, n + 2 * 3)
    assert o.get_ghosted("q").shape == (n + 6, n + 6)
    assert o.shape("q") == (n, n)


def test_mesh_rejects_non_uniform_cells():
    with pytest.raises(ValueError, match="Extent not evenly divisible"):
        Oracle(8, 8, hi=(1.0, 2.0))


def test_state_swap_and_walls_keep_zero_ghosts():
    """ProblemManagerTest.StateArrayTest analogue: after a step the Current
    array is the one advection wrote; wall ghosts are never written."""
    o = Oracle(16, 16)
    rng = np.random.default_rng(0)
    o.set("q", rng.uniform(size=(16, 16)))
    o.advect(0.01, 3)
    g = o.get_ghosted("q")
    assert not g[:3].any() and not g[-3:].any() and not g[:, :3].any() and not g[:, -3:].any()


def test_halo_encoding_across_periodic_seam():
    """ProblemManagerTest.HaloTest with one periodic rank: each ghost holds
    rank*1000 + i*100 + j*10 + 1 of the owned face it mirrors."""
    n = 10
    o = Oracle(n, n, periodic=(True, True))
    ny, nx = o.shape("u")
    gi, gj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    o.set("u", (gi + 3) * 100 + (gj + 3) * 10 + 1.0)
    o.fill_ghosts()
    g = o.get_ghosted("u")
    ey, ex = g.shape
    for j in range(ey):
        for i in range(ex):
            assert g[j, i] == ((i - 3) % nx + 3) * 100 + ((j - 3) % ny + 3) * 10 + 1


# ---- interpolation / rk3 known answers ----
@pytest.mark.parametrize("order", [1, 3])
def test_interpolation_reproduces_affine_fields(order):
    n = 32
    o = Oracle(n, n, periodic=(False, False))
    dx = 1.0 / n
    # cell centres (i + 1/2) dx: f = 2 + 3x - 5y, extended into the ghosts by fill
    ic = (np.arange(n) + 0.5) * dx
    X, Y = np.meshgrid(ic, ic, indexing="xy")
    g = o.get_ghosted("q")
    gx = (np.arange(g.shape[1]) - 3 + 0.5) * dx
    gy = (np.arange(g.shape[0]) - 3 + 0.5) * dx
    GX, GY = np.meshgrid(gx, gy, indexing="xy")
    o.set_ghosted("q", 2.0 + 3.0 * GX - 5.0 * GY)
    rng = np.random.default_rng(order)
    xy = rng.uniform(0.05, 0.95, (400, 2))
    got = o.sample("q", order, xy)
    exact = 2.0 + 3.0 * xy[:, 0] - 5.0 * xy[:, 1]
    assert np.abs(got - exact).max() < 1e-13
    o.set_ghosted("q", np.full_like(GX, 7.25))
    assert np.abs(o.sample("q", order, xy) - 7.25).max() < 1e-14


def test_cubic_bspline_at_grid_points_is_141_stencil():
    n = 16
    o = Oracle(n, n)
    rng = np.random.default_rng(3)
    g = rng.standard_normal(o.get_ghosted("q").shape)
    o.set_ghosted("q", g)
    dx = 1.0 / n
    for (i, j) in [(5, 7), (8, 8), (3, 11)]:
        x, y = (i + 0.5) * dx, (j + 0.5) * dx
        li, lj = i + 3, j + 3
        w = np.array([1.0, 4.0, 1.0]) / 6.0
        expect = sum(w[b] * w[a] * g[lj - 1 + b, li - 1 + a] for a in range(3) for b in range(3))
        got = o.sample("q", 3, np.array([[x, y]]))[0]
        assert abs(got - expect) < 1e-13


def test_rk3_uniform_velocity():
    n = 32
    o = Oracle(n, n, periodic=(True, True))
    U, V = 0.7, -0.3
    o.set("u", np.full(o.shape("u"), U))
    o.set("v", np.full(o.shape("v"), V))
    o.fill_ghosts()
    rng = np.random.default_rng(1)
    xy = rng.uniform(0.2, 0.8, (100, 2))
    dt = 0.01
    tr = o.trace(xy, dt)
    assert np.abs(tr - (xy - dt * np.array([U, V]))).max() < 1e-14


# ---- projection known answers ----
def test_streamfunction_field_is_divergence_free():
    n = 48
    rng = np.random.default_rng(2)
    psi = rng.standard_normal((n + 1, n + 1))
    psi[0] = psi[-1] = 0.0
    psi[:, 0] = psi[:, -1] = 0.0
    u, v = mac_from_streamfunction(psi, 1.0 / n, periodic=False)
    o = Oracle(n, n)
    o.set("u", u)
    o.set("v", v)
    l2, linf = o.div_norms()
    assert linf < 1e-10 * np.abs(u).max() * n


def _reference_matrix(n, dt, density, bc=(0, 0, 0, 0)):
    """initializeMatrixValues + build_matrix (src/VelocityCorrector.hpp:116-144,
    src/BoundaryConditions.hpp:57-97) as a scipy sparse matrix."""
    import scipy.sparse as sp
    dx = 1.0 / n
    scale = dt / ((density * dx) * dx)
    rows, cols, vals = [], [], []
    for gj in range(n):
        for gi in range(n):
            e = [4.0 * scale, -scale, -scale, -scale, -scale]
            if gi <= 0:
                e[1] = 0.0
                if bc[0] == 0:
                    e[0] -= scale
            if gi > n - 2:
                e[2] = 0.0
                if bc[2] == 0:
                    e[0] -= scale
            if gj <= 0:
                e[3] = 0.0
                if bc[1] == 0:
                    e[0] -= scale
            if gj > n - 2:
                e[4] = 0.0
                if bc[3] == 0:
                    e[0] -= scale
            k = gj * n + gi
            for val, (di, dj) in zip(e, [(0, 0), (-1, 0), (1, 0), (0, -1), (0, 1)]):
                if val != 0.0:
                    rows.append(k)
                    cols.append((gj + dj) * n + gi + di)
                    vals.append(val)
    return sp.csr_matrix((vals, (rows, cols)), shape=(n * n, n * n))


@pytest.mark.parametrize("bc", [(0, 0, 0, 0), (1, 1, 1, 1), (1, 0, 0, 1)])
def test_matrix_matches_build_matrix_and_is_symmetric(bc):
    n = 20
    dt, density = 0.01, 0.1
    o = Oracle(n, n, bc=bc, density=density)
    A = _reference_matrix(n, dt, density, bc)
    rng = np.random.default_rng(4)
    x = rng.standard_normal((n, n))
    y = rng.standard_normal((n, n))
    Ax = o.matvec(dt, x)
    Ay = o.matvec(dt, y)
    assert np.allclose(Ax.ravel(), A @ x.ravel(), rtol=1e-13, atol=1e-9)
    assert abs(np.vdot(x, Ay) - np.vdot(y, Ax)) <= 1e-10 * np.abs(Ax).max() * n * n
    assert abs(A - A.T).max() == 0.0


def test_cg_matches_sparse_direct_solve():
    import scipy.sparse.linalg as spla
    n = 24
    dt, density = 0.01, 0.1
    rng = np.random.default_rng(6)
    o = Oracle(n, n, bc=(1, 0, 0, 0), density=density, quirks=1)   # one FREE side: nonsingular
    u = rng.standard_normal(o.shape("u"))
    v = rng.standard_normal(o.shape("v"))
    u[:, -1] = 0.0
    v[0, :] = v[-1, :] = 0.0
    o.set("u", u)
    o.set("v", v)
    st = o.project(dt, tol=1e-13, max_iter=10000)
    assert st["status"] == 0
    b = o.get("rhs").ravel()
    A = _reference_matrix(n, dt, density, (1, 0, 0, 0))
    p_direct = spla.spsolve(A.tocsc(), b)
    p = o.get("p").ravel()
    assert np.abs(p - p_direct).max() <= 1e-9 * np.abs(p_direct).max()


def test_cg_singular_walls_matches_direct_on_mean_zero_subspace():
    import scipy.sparse.linalg as spla
    n = 16
    dt, density = 0.01, 0.1
    rng = np.random.default_rng(8)
    o = Oracle(n, n, density=density, quirks=1)
    u = rng.standard_normal(o.shape("u"))
    v = rng.standard_normal(o.shape("v"))
    u[:, 0] = u[:, -1] = 0.0
    v[0, :] = v[-1, :] = 0.0
    o.set("u", u)
    o.set("v", v)
    st = o.project(dt, tol=1e-13, max_iter=10000)
    assert st["status"] == 0
    A = _reference_matrix(n, dt, density).tolil()
    b = o.get("rhs").ravel()
    assert abs(b.sum()) < 1e-9 * np.abs(b).max()
    A[0, :] = 0.0
    A[0, 0] = 1.0            # pin one value, then compare mean-free parts
    bb = b.copy()
    bb[0] = 0.0
    p_direct = spla.spsolve(A.tocsc(), bb)
    p = o.get("p").ravel()
    d = (p - p.mean()) - (p_direct - p_direct.mean())
    assert np.abs(d).max() <= 1e-8 * np.abs(p_direct - p_direct.mean()).max()
    # Q1 fixed: the stored field's divergence is the CG residual
    assert st["div_l2"] == pytest.approx(np.sqrt(st["rr"]) / n, rel=1e-6)


def test_q1_quirk_zeroes_bottom_u_row():
    n = 16
    rng = np.random.default_rng(9)
    o = Oracle(n, n, quirks=0)
    u = rng.standard_normal(o.shape("u"))
    v = rng.standard_normal(o.shape("v"))
    u[:, 0] = u[:, -1] = 0.0
    v[0, :] = v[-1, :] = 0.0
    o.set("u", u)
    o.set("v", v)
    o.project(0.01, tol=1e-10, max_iter=5000)
    assert not o.get("u")[0].any()
    assert o.get("v")[0].any()          # wall v is not reset (src/VelocityCorrector.hpp:260)


def test_canonical_dot_matches_numpy():
    rng = np.random.default_rng(10)
    for shape in [(1, 1), (17, 33), (64, 130), (200, 257)]:
        a = rng.standard_normal(shape)
        b = rng.standard_normal(shape)
        d = oracle.canonical_dot(a, b)
        assert abs(d - float(np.sum(a * b))) <= 1e-12 * np.sum(np.abs(a * b))


def test_zero_rhs_takes_no_iterations():
    o = Oracle(16, 16)
    st = o.project(0.01)
    assert st["iterations"] == 0 and st["status"] == 0


# ---- inputs, trace and gradient known answers (the spec of Solver::_addInputs,
# TimeIntegrator::rk3 and VelocityCorrector::_applyPressure) ----
FREE, SOLID = 1, 0


def _random_state(o, rng, lo=-3.0, hi=3.0):
    q = rng.uniform(0.0, 5.0, o.shape("q"))
    u = rng.uniform(lo, hi, o.shape("u"))
    v = rng.uniform(lo, hi, o.shape("v"))
    o.set("q", q)
    o.set("u", u)
    o.set("v", v)
    return q, u, v


def test_inflow_source_tests_the_box_at_entity_positions():
    """InflowSource<2> (src/InflowSource.hpp:30-98): the half-open box
    [x0, x0+w) x [y0, y0+h) is tested at the cell centre for q and at the face
    centres for u and v; q becomes max(q, Q), a face velocity is replaced by the
    source's only where it is smaller in magnitude; not a rate."""
    n = 16
    dx = 1.0 / n
    src = ((0.25, 0.5), (0.25, 0.25), (2.0, -1.5), 3.0)
    o = Oracle(n, n, bc=(FREE,) * 4, source=src)
    rng = np.random.default_rng(21)
    q, u, v = _random_state(o, rng)
    u[8:12, 4] = u[8:12, 8] = 0.0       # faces on the box's left and right edges
    o.set("u", u)
    o.add_inputs(0.125)

    def inside(x, y):
        return (x >= 0.25) & (x < 0.5) & (y >= 0.5) & (y < 0.75)

    jc, ic = np.mgrid[0:n, 0:n]
    mq = inside((ic + 0.5) * dx, (jc + 0.5) * dx)
    eq = np.where(mq, np.maximum(q, 3.0), q)
    ju, iu = np.mgrid[0:n, 0:n + 1]
    mu = inside(iu * dx, (ju + 0.5) * dx) & (np.abs(u) < 2.0)
    eu = np.where(mu, 2.0, u)
    jv, iv = np.mgrid[0:n + 1, 0:n]
    mv = inside((iv + 0.5) * dx, jv * dx) & (np.abs(v) < 1.5)
    ev = np.where(mv, -1.5, v)
    assert np.array_equal(o.get("q"), eq)
    assert np.array_equal(o.get("u"), eu)
    assert np.array_equal(o.get("v"), ev)
    # the box's left edge (x = 0.25) is inside, its right edge (x = 0.5) outside
    assert (o.get("u")[8:12, 4] == 2.0).all()
    assert (o.get("u")[8:12, 8] == 0.0).all()


def test_body_force_adds_f_dt_on_every_face():
    """BodyForce<2> (src/BodyForce.hpp:30-69): u += f_x dt and v += f_y dt on
    every owned face, wall faces included, not scaled by the quantity."""
    n = 12
    f = (0.5, -9.81)
    dt = 0.01
    o = Oracle(n, n, bc=(FREE,) * 4, body=f)
    rng = np.random.default_rng(22)
    q, u, v = _random_state(o, rng)
    o.add_inputs(dt)
    assert np.allclose(o.get("u"), u + f[0] * dt, rtol=0, atol=1e-15)
    assert np.allclose(o.get("v"), v + f[1] * dt, rtol=0, atol=1e-15)
    assert np.array_equal(o.get("q"), q)


@pytest.mark.parametrize("bc", [(SOLID,) * 4, (SOLID, FREE, FREE, SOLID), (FREE, SOLID, SOLID, FREE)])
def test_solid_walls_zero_their_normal_faces(bc):
    """BoundaryCondition<2>::operator() (src/BoundaryConditions.hpp:102-129):
    with sides ordered [left, bottom, right, top], a SOLID side zeroes the
    normal velocity on its wall faces (u at gi = 0 or N, v at gj = 0 or N); a
    FREE side and every interior face are untouched."""
    n = 10
    o = Oracle(n, n, bc=bc)
    rng = np.random.default_rng(23)
    _, u, v = _random_state(o, rng)
    o.add_inputs(0.01)
    eu, ev = u.copy(), v.copy()
    if bc[0] == SOLID:
        eu[:, 0] = 0.0
    if bc[2] == SOLID:
        eu[:, n] = 0.0
    if bc[1] == SOLID:
        ev[0, :] = 0.0
    if bc[3] == SOLID:
        ev[n, :] = 0.0
    assert np.array_equal(o.get("u"), eu)
    assert np.array_equal(o.get("v"), ev)


@pytest.mark.parametrize("fix_q3", [False, True])
def test_rk3_third_stage_uses_v0(fix_q3):
    """TimeIntegrator::rk3 (src/TimeIntegrator.hpp:36-77) on the shear field
    u = a y, v = b x, which linear interpolation reproduces exactly: the third
    stage starts from x0 - 3/4 dt v0 (quirk Q3, :57-58); with the fix it starts
    from x0 - 3/4 dt v1 (Ralston's third-order scheme)."""
    n = 32
    dx = 1.0 / n
    a, b = 1.7, -2.3
    o = Oracle(n, n, periodic=(False, False), quirks=2 if fix_q3 else 0)
    ju, iu = np.mgrid[0:n, 0:n + 1]
    jv, iv = np.mgrid[0:n + 1, 0:n]
    o.set("u", a * (ju + 0.5) * dx)
    o.set("v", b * (iv + 0.5) * dx)
    o.fill_ghosts()

    def vel(p):
        return np.stack([a * p[:, 1], b * p[:, 0]], axis=1)

    rng = np.random.default_rng(24)
    x0 = rng.uniform(0.3, 0.7, (64, 2))
    dt = 0.05
    v0 = vel(x0)
    v1 = vel(x0 - 0.5 * dt * v0)
    v2 = vel(x0 - 0.75 * dt * (v1 if fix_q3 else v0))
    expect = x0 - dt * (2.0 / 9.0 * v0 + 3.0 / 9.0 * v1 + 4.0 / 9.0 * v2)
    got = o.trace(x0, dt)
    assert np.abs(got - expect).max() < 1e-13
    other = x0 - dt * (2.0 / 9.0 * v0 + 3.0 / 9.0 * v1
                       + 4.0 / 9.0 * vel(x0 - 0.75 * dt * (v0 if fix_q3 else v1)))
    assert np.abs(got - other).max() > 1e-7


def test_divergence_of_an_affine_field():
    """_buildRHS (src/VelocityCorrector.hpp:182-212): u = alpha x, v = beta y
    has discrete divergence alpha + beta in every cell; the L2 norm is taken
    with the cell area, so it equals |alpha + beta| on the unit box."""
    n = 24
    dx = 1.0 / n
    alpha, beta = 0.75, -2.0
    o = Oracle(n, n, bc=(FREE,) * 4)
    ju, iu = np.mgrid[0:n, 0:n + 1]
    jv, iv = np.mgrid[0:n + 1, 0:n]
    o.set("u", alpha * iu * dx)
    o.set("v", beta * jv * dx)
    l2, linf = o.div_norms()
    assert linf == pytest.approx(abs(alpha + beta), rel=1e-12)
    assert l2 == pytest.approx(abs(alpha + beta), rel=1e-12)


def test_apply_pressure_subtracts_the_face_gradient():
    """_applyPressure (src/VelocityCorrector.hpp:214-264) with SOLID walls and
    quirk Q1 kept: every owned face gets u -= dt/(rho dx) (p(i) - p(i-1)),
    physical ghosts of p are 0, so the bottom wall's v becomes
    v - scale p(i, 0) and the top wall's v + scale p(i, N-1); u's bottom row is
    then zeroed by the J-face condition applied to u (:260)."""
    n = 16
    dx = 1.0 / n
    dt, rho = 0.02, 1.3
    o = Oracle(n, n, density=rho)
    rng = np.random.default_rng(25)
    _, u, v = _random_state(o, rng)
    o.project(dt, tol=1e-10, max_iter=5000)
    p = o.get("p")
    s = dt / (rho * dx)
    pz = np.zeros((n + 2, n + 2))
    pz[1:-1, 1:-1] = p
    eu = u - s * (pz[1:-1, 1:] - pz[1:-1, :-1])
    ev = v - s * (pz[1:, 1:-1] - pz[:-1, 1:-1])
    eu[:, 0] = 0.0          # I-face condition on the SOLID left and right walls
    eu[:, n] = 0.0
    eu[0, :] = 0.0          # Q1: the J-face condition applied to u
    tol = 1e-12 * (np.abs(u).max() + s * np.abs(p).max())
    assert np.abs(o.get("u") - eu).max() <= tol
    assert np.abs(o.get("v") - ev).max() <= tol
    vn = o.get("v")
    assert np.abs(vn[0] - (v[0] - s * p[0])).max() <= tol
    assert np.abs(vn[n] - (v[n] + s * p[n - 1])).max() <= tol
