"""FP64 parity of the CUDA path against the CPU oracle, through the C ABI.

The FP64 kernels and the oracle follow the same evaluation order (explicit
fma, fixed reduction order), so every comparison here is bit for bit.
"""
import numpy as np
import pytest

from helpers import FIELDS, assert_fields_equal, load_state, make_pair, opts, random_state

pytestmark = pytest.mark.gpu

SHAPES = [(16, 16), (33, 20), (64, 64), (130, 70)]
INFLOW = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)


@pytest.mark.parametrize("nx,ny", SHAPES)
@pytest.mark.parametrize("periodic", [(False, False), (True, True), (True, False)])
def test_interpolation_points(built, nx, ny, periodic):
    rng = np.random.default_rng(nx * 7 + ny)
    o, c = make_pair(nx, ny, periodic=periodic)
    load_state(o, c, random_state(o, rng))
    o.fill_ghosts()
    c.fill_ghosts()
    h = ny / nx
    xy = np.stack([rng.uniform(-0.05, 1.05, 500), rng.uniform(-0.05 * h, 1.05 * h, 500)], axis=1)
    for f in FIELDS:
        for order in (1, 3):
            a = o.sample(f, order, xy)
            b = c.interp_points(f, order, xy)
            assert np.array_equal(a, b), (f, order, np.abs(a - b).max())


@pytest.mark.parametrize("nx,ny", SHAPES[:3])
def test_rk3_trace(built, nx, ny):
    rng = np.random.default_rng(5)
    o, c = make_pair(nx, ny)
    load_state(o, c, random_state(o, rng))
    xy = np.stack([rng.uniform(0, 1, 300), rng.uniform(0, ny / nx, 300)], axis=1)
    dt = 0.3 / nx
    assert np.array_equal(o.trace(xy, dt), c.trace_points(xy, dt))


@pytest.mark.parametrize("periodic", [(True, True), (True, False), (False, True)])
def test_ghost_fill_matches_oracle(built, periodic):
    rng = np.random.default_rng(11)
    o, c = make_pair(24, 18, periodic=periodic)
    load_state(o, c, random_state(o, rng))
    o.fill_ghosts()
    c.fill_ghosts()
    for f in FIELDS:
        assert np.array_equal(o.get_ghosted(f), c.download_ghosted(f)), f


def test_halo_encoding_periodic(built):
    """tests/tstProblemManager.cpp:61-98 with one periodic rank: every ghost
    holds the encoding rank*1000 + i*100 + j*10 + 1 of the owned face it
    mirrors (local indices of the owner)."""
    n = 12
    o, c = make_pair(n, n, periodic=(True, True))
    ny, nx = c.owned_shape("u")
    gi, gj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    enc = (gi + 3) * 100 + (gj + 3) * 10 + 1.0
    c.upload("u", enc)
    c.fill_ghosts()
    g = c.download_ghosted("u")
    ey, ex = g.shape
    for j in range(ey):
        for i in range(ex):
            si = (i - 3) % nx + 3
            sj = (j - 3) % ny + 3
            assert g[j, i] == si * 100 + sj * 10 + 1


@pytest.mark.parametrize("nx,ny", SHAPES)
@pytest.mark.parametrize("order", [1, 3])
@pytest.mark.parametrize("periodic", [(False, False), (True, True)])
def test_advect_step(built, nx, ny, order, periodic):
    rng = np.random.default_rng(nx + 3 * ny + order)
    o, c = make_pair(nx, ny, periodic=periodic)
    st = random_state(o, rng, scale=0.5)
    load_state(o, c, st)
    dt = 0.4 / nx
    o.advect(dt, order)
    c.advect(dt, order)
    assert_fields_equal(o, c, tag="advect")


@pytest.mark.parametrize("quirks", [0, 1, 2, 3])
def test_advect_quirks(built, quirks):
    rng = np.random.default_rng(quirks)
    o, c = make_pair(40, 40, quirks=quirks)
    load_state(o, c, random_state(o, rng, scale=0.5))
    o.advect(0.01, 3)
    c.advect(0.01, 3)
    assert_fields_equal(o, c, tag=f"quirks={quirks}")


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("density_scaled", [False, True])
@pytest.mark.parametrize("bc", [(0, 0, 0, 0), (1, 0, 1, 0), (0, 1, 1, 0)])
def test_add_inputs(built, mode, density_scaled, bc):
    rng = np.random.default_rng(mode + 2 * density_scaled)
    o, c = make_pair(48, 48, bc=bc, source=((0.3, 0.2), (0.25, 0.3), (2.0, -1.5), 0.7), source_mode=mode,
                     body=(0.5, -9.8), body_density_scaled=density_scaled)
    load_state(o, c, random_state(o, rng))
    o.add_inputs(0.004)
    c.add_inputs(0.004)
    assert_fields_equal(o, c, tag="inputs")


@pytest.mark.parametrize("nx,ny", SHAPES)
@pytest.mark.parametrize("periodic", [(False, False), (True, True), (False, True)])
@pytest.mark.parametrize("quirks", [0, 1])
def test_project(built, nx, ny, periodic, quirks):
    rng = np.random.default_rng(nx * ny + quirks)
    o, c = make_pair(nx, ny, periodic=periodic, quirks=quirks)
    load_state(o, c, random_state(o, rng))
    dt = 0.5 / nx
    so = o.project(dt, tol=1e-9, max_iter=5000)
    sg = c.project(dt, opts(tol=1e-9, max_iter=5000))
    assert so["status"] == sg["status"] == 0
    assert so["iterations"] == sg["iterations"]
    assert so["bb"] == sg["b_norm"] ** 2 or np.sqrt(so["bb"]) == sg["b_norm"]
    assert np.sqrt(so["rr"]) == sg["r_norm"]
    assert so["div_l2"] == sg["div_l2"] and so["div_linf"] == sg["div_linf"]
    assert np.array_equal(o.get("p"), c.download("p"))
    assert_fields_equal(o, c, fields=("u", "v"), tag="project")


@pytest.mark.parametrize("bc", [(1, 1, 1, 1), (1, 0, 0, 0), (0, 0, 1, 1)])
def test_project_free_boundaries(built, bc):
    rng = np.random.default_rng(sum(bc))
    o, c = make_pair(50, 36, bc=bc)
    load_state(o, c, random_state(o, rng))
    so = o.project(0.01, tol=1e-10, max_iter=5000)
    sg = c.project(0.01, opts(tol=1e-10, max_iter=5000))
    assert so["iterations"] == sg["iterations"] and so["status"] == sg["status"] == 0
    assert np.array_equal(o.get("p"), c.download("p"))
    assert_fields_equal(o, c, fields=("u", "v"))


def test_project_unpreconditioned(built):
    rng = np.random.default_rng(9)
    o, c = make_pair(40, 40, precon_none=True)
    load_state(o, c, random_state(o, rng))
    so = o.project(0.01, tol=1e-8, max_iter=5000)
    sg = c.project(0.01, opts(tol=1e-8, max_iter=5000, precon="None"))
    assert so["iterations"] == sg["iterations"]
    assert np.array_equal(o.get("p"), c.download("p"))


def test_project_abs_tol(built):
    rng = np.random.default_rng(21)
    o, c = make_pair(64, 64, periodic=(True, True))
    load_state(o, c, random_state(o, rng))
    so = o.project(0.01, tol=0.0, abs_tol=1e-7, max_iter=5000)
    sg = c.project(0.01, opts(tol=0.0, abs_tol=1e-7, max_iter=5000))
    assert so["iterations"] == sg["iterations"] and sg["status"] == 0
    assert sg["div_l2"] <= 1e-7 * (1 + 1e-12)
    assert np.array_equal(o.get("p"), c.download("p"))


@pytest.mark.parametrize("n,steps,order", [(32, 12, 1), (64, 8, 3), (256, 3, 1)])
def test_full_steps_config0(built, n, steps, order):
    """Solver::setup + Solver::step (src/Solver.hpp:125-147) from a zero state
    with the config-0 inflow, bit for bit over several steps."""
    o, c = make_pair(n, n, source=INFLOW, density=0.1)
    dt = 0.5 * (1.0 / n) / 3.0
    so = o.setup(dt, tol=1e-8, max_iter=20000)
    sg = c.setup(dt, opts(tol=1e-8, max_iter=20000))
    assert so["iterations"] == sg["iterations"]
    for k in range(steps):
        so = o.step(dt, order, tol=1e-8, max_iter=20000)
        sg = c.step(dt, order, opts(tol=1e-8, max_iter=20000))
        assert so["iterations"] == sg["iterations"], k
        assert sg["status"] == 0
    assert_fields_equal(o, c, tag=f"after {steps} steps")
    assert np.array_equal(o.get("p"), c.download("p"))


def test_full_steps_buoyancy_periodic_x(built):
    o, c = make_pair(48, 48, periodic=(True, False), source=INFLOW, body=(0.0, -9.8), body_density_scaled=True,
                     quirks=0)
    dt = 0.5 / 48 / 3.0
    rng = np.random.default_rng(4)
    st = random_state(o, rng, scale=0.1)
    st["v"][0, :] = 0.0
    st["v"][-1, :] = 0.0
    load_state(o, c, st)
    for k in range(6):
        so = o.step(dt, 3, tol=1e-9, max_iter=20000)
        sg = c.step(dt, 3, opts(tol=1e-9, max_iter=20000))
        assert so["iterations"] == sg["iterations"], k
    assert_fields_equal(o, c)
