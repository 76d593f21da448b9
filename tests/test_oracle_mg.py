"""CPU checks of the oracle's multigrid preconditioner: the V-cycle is a
symmetric positive-definite operator (CG needs both), the level hierarchy
follows the coarsening rule, and MG-PCG reaches the Jacobi-PCG solution."""
import numpy as np
import pytest

from oracle import Oracle

CASES = [
    (64, 64, (False, False), (0, 0, 0, 0), 4),
    (48, 40, (False, False), (0, 1, 1, 0), 3),
    (33, 31, (False, False), (0, 0, 0, 0), 1),
    (64, 32, (True, True), (0, 0, 0, 0), 3),
    (36, 36, (True, False), (0, 0, 0, 0), 2),
]


@pytest.mark.parametrize("nx,ny,periodic,bc,levels", CASES)
def test_vcycle_symmetric_positive(nx, ny, periodic, bc, levels):
    o = Oracle(nx, ny, hi=(1.0, ny / nx), periodic=periodic, bc=bc, precon_mg=True, density=0.1)
    rng = np.random.default_rng(nx + ny)
    r1, r2 = rng.standard_normal((2, ny, nx))
    z1, nlev = o.mg_apply(0.01, r1)
    z2, _ = o.mg_apply(0.01, r2)
    assert nlev == levels
    a, b = float((z1 * r2).sum()), float((r1 * z2).sum())
    assert abs(a - b) <= 1e-12 * abs(a)
    assert (z1 * r1).sum() > 0 and (z2 * r2).sum() > 0


def test_vcycle_linear():
    o = Oracle(64, 64, precon_mg=True, density=0.1)
    rng = np.random.default_rng(3)
    r1, r2 = rng.standard_normal((2, 64, 64))
    z1, _ = o.mg_apply(0.01, r1)
    z2, _ = o.mg_apply(0.01, r2)
    z12, _ = o.mg_apply(0.01, 2.0 * r1 + r2)
    assert np.allclose(z12, 2.0 * z1 + z2, rtol=0, atol=1e-12 * np.abs(z12).max())


def _state(o, rng):
    ny, nx = o.shape("q")
    st = {"q": rng.uniform(0, 1, (ny, nx)), "u": rng.standard_normal(o.shape("u")),
          "v": rng.standard_normal(o.shape("v"))}
    st["u"][:, 0] = st["u"][:, -1] = 0.0
    st["v"][0, :] = st["v"][-1, :] = 0.0
    return st


@pytest.mark.parametrize("bc", [(0, 0, 0, 0), (1, 0, 0, 1)])
def test_mg_pcg_matches_jacobi_solution(bc):
    # quirk Q1 fixed: otherwise the wall rows of v keep p's null-space
    # constant (the J-face wall condition lands on u), which depends on the solver
    rng = np.random.default_rng(5)
    oj = Oracle(64, 64, bc=bc, density=0.1, quirks=1)
    om = Oracle(64, 64, bc=bc, density=0.1, precon_mg=True, quirks=1)
    st = _state(oj, rng)
    for f in ("q", "u", "v"):
        oj.set(f, st[f])
        om.set(f, st[f])
    sj = oj.project(0.01, tol=1e-11, max_iter=5000)
    sm = om.project(0.01, tol=1e-11, max_iter=5000)
    assert sj["status"] == sm["status"] == 0
    assert sm["iterations"] * 10 < sj["iterations"]
    for f in ("u", "v"):
        assert np.abs(oj.get(f) - om.get(f)).max() < 1e-8


def test_mg_odd_periodic_rejected():
    with pytest.raises(ValueError, match="even"):
        Oracle(33, 32, hi=(1.0, 32 / 33), periodic=(True, False), precon_mg=True)
