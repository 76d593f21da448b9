"""The mixed pressure gradient's unit-per-warp kernel against the per-face one.

A mixed context subtracts the pressure gradient from the velocity pairs in
k_apply_pairs (one warp per 64 x 16 cells, the faces of the owned cells)
plus, on a walled axis, k_apply_edges (the faces past the last cell);
cf_test_apply_general sends every face through k_apply_pressure, the
one-thread-per-face kernel of the FP64 gradient.  Both must give the same
bits: whole mixed steps (graphs and direct launches), odd and small grids,
every wall rule (solid and free walls, the Q1 quirk fixed and not) and the
adjoint's transposed projection are compared bit for bit.  On a grid
periodic along both axes the gradient kernel also takes the divergence norms
of its result (k_apply_pairs_norms); they must equal k_div_norms' bit for bit.
"""
import numpy as np
import pytest

from cajitafluids_gb300 import Context, SolverOptions
from cajitafluids_gb300 import _lib as L
from cajitafluids_gb300.workloads import gaussian_blobs, spectral_velocity

pytestmark = pytest.mark.gpu

FIELDS = ("q", "u", "v")


def _ctx(nx, ny, periodic, bc, quirks, general, graphs=True):
    c = Context(nx, ny, hi=(1.0, ny / nx), periodic=periodic, precision="mixed")
    c.set_bc(bc)
    c.set_density(0.1)
    c.set_quirks(quirks)
    c.set_body_force((0.0, -9.8), False)
    c.set_graphs(graphs)
    assert c.lib.cf_test_apply_general(c.h, general) == L.CF_OK
    return c


def _state(nx, ny, periodic, seed):
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((ny, nx if periodic[0] else nx + 1))
    v = rng.standard_normal((ny if periodic[1] else ny + 1, nx))
    if not periodic[0]:
        u[:, 0] = u[:, -1] = 0.0
    if not periodic[1]:
        v[0, :] = v[-1, :] = 0.0
    q = rng.uniform(0.0, 1.0, (ny, nx))
    return {"q": q, "u": u, "v": v}


@pytest.mark.parametrize("nx,ny,periodic", [(96, 80, (True, True)), (70, 45, (False, False)),
                                            (33, 65, (True, False)), (65, 33, (False, True)),
                                            (8, 8, (False, False))])
@pytest.mark.parametrize("bc,quirks", [((0, 0, 0, 0), 0), ((0, 0, 0, 0), L.CF_FIX_Q1),
                                       ((1, 0, 1, 1), 0), ((0, 1, 0, 0), L.CF_FIX_Q1)])
@pytest.mark.parametrize("graphs", [True, False])
def test_unit_gradient_equals_per_face_gradient(nx, ny, periodic, bc, quirks, graphs):
    s = _state(nx, ny, periodic, seed=nx * 3 + ny)
    dt = 0.4 / max(nx, ny) / max(np.abs(s["u"]).max(), np.abs(s["v"]).max())
    # the multigrid wants an even cell count along a periodic axis
    odd = (periodic[0] and nx % 2) or (periodic[1] and ny % 2)
    o = SolverOptions(tol=1e-10, max_iter=20000, precon="Diagonal" if odd else "PFMG")
    out = []
    for general in (0, 1):
        c = _ctx(nx, ny, periodic, bc, quirks, general, graphs)
        for f in FIELDS:
            c.upload(f, s[f])
        norms = []
        for _ in range(3):
            r = c.step(dt, 3, o)
            norms.append((r["div_l2"], r["div_linf"]))
        out.append({f: c.download(f) for f in FIELDS})
        out[-1]["norms"] = norms
    for f in FIELDS:
        a, b = out[0][f], out[1][f]
        assert np.array_equal(a, b), (f, np.count_nonzero(a != b))
    # periodic both ways: the norms come from the gradient kernel itself
    assert out[0]["norms"] == out[1]["norms"]


@pytest.mark.parametrize("periodic", [False, True])
def test_unit_gradient_in_the_adjoint(periodic):
    n = 48
    u, v = spectral_velocity(n, 3, periodic, kmax=6)
    q = gaussian_blobs(n, 4, count=4, sigma=0.08)
    dt = 0.4 / n / max(np.abs(u).max(), np.abs(v).max())
    y = np.random.default_rng(1).standard_normal(q.shape)
    o = SolverOptions(tol=1e-10, max_iter=20000, precon="PFMG")
    grads = []
    for general in (0, 1):
        c = _ctx(n, n, (periodic, periodic), (0, 0, 0, 0), L.CF_FIX_Q1, general)
        for f, a in (("q", q), ("u", 0.6 * u), ("v", 0.6 * v)):
            c.upload(f, a)
        c.forward_checkpointed(6, 3, dt, 3, o)
        grads.append(c.backward(y))
    for f in FIELDS:
        assert np.array_equal(grads[0][f], grads[1][f]), f
