"""Multigrid-preconditioned CG (the PFMG / SMG preconditioner names of
src/VelocityCorrector.hpp:324-338) on the GPU against the oracle's MG-PCG.

FP64: the V-cycle kernels follow the oracle's operation order (explicit fma,
colour-ordered Gauss-Seidel half sweeps, fixed restriction and prolongation
sums) and the CG scalars use the canonical reductions, so pressure,
velocities and iteration counts agree bit for bit.  Mixed precision: FP32
V-cycle inside the FP32 inner CG with FP64 reliable updates; checked against
the FP64 oracle through the divergence it leaves and the velocity error.
"""
import numpy as np
import pytest

from cajitafluids_gb300 import CfError
from helpers import assert_fields_equal, load_state, make_pair, opts, random_state

pytestmark = pytest.mark.gpu

INFLOW = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)

# (nx, ny, periodic, bc): power-of-two, ragged, single-level odd, periodic in
# one and both axes, coarsest levels too large for the one-CTA bottom solver
# (65^2 and 130^2 -> 65^2), and a deep hierarchy (512^2 -> 8^2)
CASES = [
    (64, 64, (False, False), (0, 0, 0, 0)),
    (48, 40, (False, False), (0, 1, 1, 0)),
    (33, 31, (False, False), (0, 0, 0, 0)),
    (98, 98, (False, False), (1, 0, 0, 1)),
    (64, 32, (True, True), (0, 0, 0, 0)),
    (72, 36, (True, False), (0, 0, 0, 0)),
    (256, 128, (False, False), (0, 0, 0, 0)),
    (65, 65, (False, False), (0, 0, 0, 0)),
    (130, 130, (False, False), (0, 1, 0, 0)),
    (512, 512, (True, True), (0, 0, 0, 0)),
]


@pytest.mark.parametrize("fused", ["1", "0"])
@pytest.mark.parametrize("nx,ny,periodic,bc", CASES)
def test_project_mg_bitwise(built, monkeypatch, nx, ny, periodic, bc, fused):
    """Both forms of the levels above the one-CTA bottom solver: the fused
    pre/post kernels (default) and one launch per half sweep (CF_MG_FUSED=0)."""
    monkeypatch.setenv("CF_MG_FUSED", fused)
    rng = np.random.default_rng(nx * 3 + ny)
    o, c = make_pair(nx, ny, periodic=periodic, bc=bc, precon_mg=True)
    load_state(o, c, random_state(o, rng))
    dt = 0.5 / nx
    so = o.project(dt, tol=1e-10, max_iter=500)
    sg = c.project(dt, opts(tol=1e-10, max_iter=500, precon="PFMG"))
    assert so["status"] == sg["status"] == 0
    assert so["iterations"] == sg["iterations"]
    assert so["iterations"] < 60
    assert np.sqrt(so["rr"]) == sg["r_norm"]
    assert so["div_l2"] == sg["div_l2"] and so["div_linf"] == sg["div_linf"]
    assert np.array_equal(o.get("p"), c.download("p"))
    assert_fields_equal(o, c, fields=("u", "v"), tag="mg project")


@pytest.mark.parametrize("name", ["PFMG", "SMG", "MG"])
def test_mg_names_same_solver(built, name):
    rng = np.random.default_rng(2)
    o, c = make_pair(40, 40, precon_mg=True)
    load_state(o, c, random_state(o, rng))
    so = o.project(0.01, tol=1e-9, max_iter=500)
    sg = c.project(0.01, opts(tol=1e-9, max_iter=500, precon=name))
    assert so["iterations"] == sg["iterations"]
    assert np.array_equal(o.get("p"), c.download("p"))


def test_full_steps_config0_mg(built):
    """Solver::setup + Solver::step with the reference CLI's default
    PCG + PFMG pairing (examples/advection.cpp:186-189), bit for bit."""
    n = 64
    o, c = make_pair(n, n, source=INFLOW, density=0.1, precon_mg=True)
    dt = 0.5 * (1.0 / n) / 3.0
    so = o.setup(dt, tol=1e-8, max_iter=500)
    sg = c.setup(dt, opts(tol=1e-8, max_iter=500, precon="PFMG"))
    assert so["iterations"] == sg["iterations"]
    for k in range(6):
        so = o.step(dt, 3, tol=1e-8, max_iter=500)
        sg = c.step(dt, 3, opts(tol=1e-8, max_iter=500, precon="PFMG"))
        assert so["iterations"] == sg["iterations"], k
        assert sg["status"] == 0
    assert_fields_equal(o, c, tag="mg steps")
    assert np.array_equal(o.get("p"), c.download("p"))


def test_full_steps_config1_size(built):
    """The 1024^2 workload with all walls SOLID, the config-0 inflow, gravity
    scaled by the quantity (extension Q5), cubic values and tol 1e-10: setup
    and three steps bit for bit, with the divergence norms of every step."""
    n = 1024
    o, c = make_pair(n, n, source=INFLOW, body=(0.0, -9.8), body_density_scaled=True, density=0.1,
                     precon_mg=True)
    dt = 0.5 * (1.0 / n) / 3.0
    so = o.setup(dt, tol=1e-10, max_iter=500)
    sg = c.setup(dt, opts(tol=1e-10, max_iter=500, precon="PFMG"))
    assert so["iterations"] == sg["iterations"]
    for k in range(3):
        so = o.step(dt, 3, tol=1e-10, max_iter=500)
        sg = c.step(dt, 3, opts(tol=1e-10, max_iter=500, precon="PFMG"))
        assert sg["status"] == 0 and so["iterations"] == sg["iterations"], k
        assert so["div_l2"] == sg["div_l2"] and so["div_linf"] == sg["div_linf"], k
    assert_fields_equal(o, c, tag="1024^2 steps")
    assert np.array_equal(o.get("p"), c.download("p"))


def test_mg_max_iter_and_zero_rhs(built):
    rng = np.random.default_rng(8)
    o, c = make_pair(64, 64, precon_mg=True)
    load_state(o, c, random_state(o, rng))
    so = o.project(0.01, tol=1e-14, max_iter=3)
    sg = c.project(0.01, opts(tol=1e-14, max_iter=3, precon="PFMG"))
    assert so["status"] == sg["status"] == 1 and sg["iterations"] == 3
    assert np.array_equal(o.get("p"), c.download("p"))
    # a divergence-free state converges at once (b = 0)
    o2, c2 = make_pair(32, 32, precon_mg=True)
    z = {f: np.zeros(o2.shape(f)) for f in ("q", "u", "v")}
    load_state(o2, c2, z)
    sg = c2.project(0.01, opts(tol=1e-8, precon="PFMG"))
    assert sg["status"] == 0 and sg["iterations"] == 0


def test_mg_odd_periodic_rejected(built):
    from cajitafluids_gb300 import Context
    c = Context(33, 32, hi=(1.0, 32 / 33), periodic=(True, False))
    with pytest.raises(CfError) as e:
        c.project(0.01, opts(precon="PFMG"))
    assert "even" in str(e.value)


@pytest.mark.parametrize("nx,ny,periodic", [(128, 128, (False, False)), (96, 64, (True, True))])
def test_mixed_mg(built, nx, ny, periodic):
    rng = np.random.default_rng(nx + ny)
    o, c = make_pair(nx, ny, periodic=periodic, precision="mixed", precon_mg=True)
    st = random_state(o, rng)
    load_state(o, c, st)
    dt = 0.5 / nx
    so = o.project(dt, tol=1e-9, max_iter=500)
    sg = c.project(dt, opts(tol=1e-9, max_iter=500, precon="PFMG"))
    assert sg["status"] == 0
    assert sg["iterations"] <= 3 * so["iterations"] + 10
    assert sg["r_norm"] <= 1e-9 * sg["b_norm"] * (1 + 1e-9)
    for f in ("u", "v"):
        a, b = o.get(f), c.download(f)
        assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max(), f


def test_mixed_mg_steps(built):
    n = 128
    o, c = make_pair(n, n, source=INFLOW, density=0.1, precision="mixed", precon_mg=True)
    dt = 0.5 * (1.0 / n) / 3.0
    o.setup(dt, tol=1e-8, max_iter=500)
    c.setup(dt, opts(tol=1e-8, max_iter=500, precon="PFMG"))
    for k in range(4):
        o.step(dt, 3, tol=1e-8, max_iter=500)
        sg = c.step(dt, 3, opts(tol=1e-8, max_iter=500, precon="PFMG"))
        assert sg["status"] == 0, k
    for f in ("u", "v"):
        a, b = o.get(f), c.download(f)
        assert np.abs(a - b).max() <= 1e-4 * max(np.abs(a).max(), 1e-30), f
    qa, qb = o.get("q"), c.download("q")
    assert np.abs(qa - qb).max() <= 1e-4


def _mixed_mg_run(nx, ny, periodic, bc, strips, monkeypatch, seed, rz_fused="0"):
    from cajitafluids_gb300 import Context
    monkeypatch.setenv("CF_MG_STRIPS", strips)
    monkeypatch.setenv("CF_MG_RZ_FUSED", rz_fused)
    rng = np.random.default_rng(seed)
    shapes = {"q": (ny, nx), "u": (ny, nx + (0 if periodic[0] else 1)), "v": (ny + (0 if periodic[1] else 1), nx)}
    c = Context(nx, ny, hi=(1.0, ny / nx), periodic=periodic, precision="mixed")
    c.set_bc(bc)
    for f, shp in shapes.items():
        c.upload(f, rng.standard_normal(shp))
    st = [c.project(0.5 / nx, opts(tol=1e-9, max_iter=60, precon="PFMG"))]
    st.append(c.project(0.5 / nx, opts(tol=1e-11, max_iter=60, precon="PFMG")))
    out = {f: c.download(f) for f in ("p", "u", "v")}
    c.close()
    return st, out


@pytest.mark.parametrize("nx,ny,periodic,bc", [
    (2048, 1024, (True, True), (0, 0, 0, 0)),
    (2100, 1100, (False, False), (0, 1, 0, 1)),
    (2176, 1088, (True, False), (1, 0, 1, 0)),
    (4096, 2048, (True, True), (0, 0, 0, 0)),
])
def test_mixed_mg_register_strips(built, monkeypatch, nx, ny, periodic, bc):
    """The FP32 register strips (interior of the large levels) and the tile
    kernels compute identical V-cycles: projections with strips of 32 and 8
    rows equal those with tiles only (CF_MG_STRIPS=0) bit for bit.  r.z is
    formed by its own kernel here (CF_MG_RZ_FUSED=0): the fused form sums in
    an order that follows the tiling."""
    ref_st, ref = _mixed_mg_run(nx, ny, periodic, bc, "0", monkeypatch, nx + ny)
    assert ref_st[0]["iterations"] > 2
    for strips in ("32", "8"):
        st, out = _mixed_mg_run(nx, ny, periodic, bc, strips, monkeypatch, nx + ny)
        for a, b in zip(ref_st, st):
            assert a["status"] == b["status"] and a["iterations"] == b["iterations"], strips
            assert a["r_norm"] == b["r_norm"], strips
        for f in ("p", "u", "v"):
            assert np.array_equal(ref[f], out[f]), (strips, f)


@pytest.mark.parametrize("nx,ny,periodic,bc", [
    (2048, 1024, (True, True), (0, 0, 0, 0)),
    (2100, 1100, (False, False), (0, 1, 0, 1)),
    (200, 136, (True, False), (0, 0, 0, 1)),
    (96, 64, (True, True), (0, 0, 0, 0)),
])
def test_mixed_mg_rz_fused(built, monkeypatch, nx, ny, periodic, bc):
    """r.z, the CG scalars and z's periodic ghosts formed by the finest
    post-smoothing kernel (default) agree with the separate kernels up to the
    order of the FP32 sums: same iteration counts (within one), same
    projected velocities to FP32 accuracy."""
    ref_st, ref = _mixed_mg_run(nx, ny, periodic, bc, "32", monkeypatch, nx + ny, rz_fused="0")
    st, out = _mixed_mg_run(nx, ny, periodic, bc, "32", monkeypatch, nx + ny, rz_fused="1")
    for a, b in zip(ref_st, st):
        assert a["status"] == b["status"]
        assert abs(a["iterations"] - b["iterations"]) <= 1
    for f in ("u", "v"):
        d = np.abs(ref[f] - out[f]).max()
        assert d <= 1e-6 * np.abs(ref[f]).max(), (f, d)


@pytest.mark.parametrize("nx,ny,periodic,bc", [
    (256, 256, (True, True), (0, 0, 0, 0)),
    (192, 128, (False, False), (0, 1, 0, 1)),
])
def test_mixed_mg_update_every_iteration(built, nx, ny, periodic, bc):
    """Reliable-update threshold >= 0.5: the inner step only advances x and
    every iteration ends with the double-float residual.  Same results, bit
    for bit, as the full inner step at a threshold just below 0.5 whenever
    that run also updated after every iteration."""
    from cajitafluids_gb300 import Context
    rng = np.random.default_rng(nx * ny)
    shapes = {"q": (ny, nx), "u": (ny, nx + (0 if periodic[0] else 1)), "v": (ny + (0 if periodic[1] else 1), nx)}
    state = {f: rng.standard_normal(shp) for f, shp in shapes.items()}
    runs = []
    for itol in (0.49, 0.5):
        c = Context(nx, ny, hi=(1.0, ny / nx), periodic=periodic, precision="mixed")
        c.set_bc(bc)
        for f, a in state.items():
            c.upload(f, a)
        st = c.project(0.5 / nx, opts(tol=1e-9, max_iter=200, precon="PFMG", inner_tol=itol))
        runs.append((st, {f: c.download(f) for f in ("p", "u", "v")}))
        c.close()
    (sa, fa), (sb, fb) = runs
    assert sb["status"] == 0 and sb["outer_iterations"] >= sb["iterations"]
    assert sa["outer_iterations"] >= sa["iterations"], "the comparison run did not update every iteration"
    assert sa["iterations"] == sb["iterations"] and sa["r_norm"] == sb["r_norm"]
    for f in ("p", "u", "v"):
        assert np.array_equal(fa[f], fb[f]), f
