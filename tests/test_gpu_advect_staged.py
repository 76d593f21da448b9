"""The FP32 advection's shared-memory windows against its global-memory path.

Each 32 x 32 tile of the mixed-precision advection copies the u, v and q
windows its traces read into shared memory when (dt / dx) max|u, v| over the
window is at most 0.99, and otherwise reads global memory with the clamped
stencil.  Both must give the same bits: cf_test_advect_unstaged sends every
tile down the global path, and the results are compared bit for bit, with
every tile staged (the bench's CFL of 0.5) and with a fast blob that sends
some tiles to the global path in the same launch.
"""
import numpy as np
import pytest

from cajitafluids_gb300 import Context, SolverOptions
from cajitafluids_gb300 import _lib as L
from cajitafluids_gb300.workloads import spectral_scalar, spectral_velocity

pytestmark = pytest.mark.gpu

FIELDS = ("q", "u", "v")


def _pair(nx, ny, periodic, bc=(0, 0, 0, 0), source=None, source_mode=0, body=(0.0, 0.0), quirks=0):
    cs = []
    for unstaged in (0, 1):
        c = Context(nx, ny, hi=(1.0, ny / nx), periodic=periodic, precision="mixed")
        c.set_bc(bc)
        if source is not None:
            c.set_source(*source, source_mode)
        c.set_body_force(body, False)
        c.set_density(0.1)
        c.set_quirks(quirks)
        assert c.lib.cf_test_advect_unstaged(c.h, unstaged) == L.CF_OK
        cs.append(c)
    return cs


def _state(nx, ny, periodic, seed, blob=0.0):
    rng = np.random.default_rng(seed)
    shp_u = (ny, nx if periodic[0] else nx + 1)
    shp_v = (ny if periodic[1] else ny + 1, nx)
    u = rng.standard_normal(shp_u)
    v = rng.standard_normal(shp_v)
    if blob:
        # a fast patch near one corner: the tiles around it exceed the window
        u[: ny // 5, : nx // 5] *= blob
        v[: ny // 5, : nx // 5] *= blob
    if not periodic[0]:
        u[:, 0] = u[:, -1] = 0.0
    if not periodic[1]:
        v[0, :] = v[-1, :] = 0.0
    q = rng.uniform(0.0, 1.0, (ny, nx))
    return {"q": q, "u": u, "v": v}


def _same(cs):
    for f in FIELDS:
        a, b = cs[0].download(f), cs[1].download(f)
        assert np.array_equal(a, b), (f, np.count_nonzero(a != b), float(np.abs(a - b).max()))


@pytest.mark.parametrize("nx,ny,periodic", [(96, 80, (True, True)), (70, 45, (False, False)),
                                            (33, 65, (True, False)), (8, 8, (False, True))])
@pytest.mark.parametrize("order", [1, 3])
@pytest.mark.parametrize("blob", [0.0, 6.0])
def test_staged_advection_equals_global_path(built, nx, ny, periodic, order, blob):
    s = _state(nx, ny, periodic, seed=nx * 7 + ny + order, blob=blob)
    umax = max(np.abs(s["u"]).max(), np.abs(s["v"]).max())
    dx = 1.0 / nx
    # CFL 0.5 on the slow part; with the blob its tiles move up to about 3 cells
    dt = 0.5 * dx / (umax / (blob if blob else 1.0))
    cs = _pair(nx, ny, periodic)
    for c in cs:
        for f in FIELDS:
            c.upload(f, s[f])
        c.advect(dt, order)
    _same(cs)


@pytest.mark.parametrize("quirks", [0, 2])
def test_staged_steps_with_inputs_equal_global_path(built, quirks):
    """Whole mixed steps on a walled grid with the inflow box (clamp form) and
    gravity, so the fused inputs epilogue runs on both paths."""
    n = 64
    u, v = spectral_velocity(n, 5, False, kmax=8)
    q = spectral_scalar(n, 6, kmax=8)
    src = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)
    cs = _pair(n, n, (False, False), source=src, body=(0.0, -9.8), quirks=quirks)
    dt = 0.5 / n / 3.0
    o = SolverOptions(tol=1e-10, max_iter=20000, precon="PFMG")
    for c in cs:
        for f, a in (("q", q), ("u", u), ("v", v)):
            c.upload(f, a)
        c.setup(dt, o)
        for _ in range(4):
            c.step(dt, 3, o)
    _same(cs)
