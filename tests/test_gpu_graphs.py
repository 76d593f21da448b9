"""Launch modes: the pressure solve through CUDA graphs (device-resident
projection graph; the default) and with every kernel launched on its own
(cf_set_graphs(ctx, 0), host-polled) give the same bits, in FP64 and mixed
precision, with the Jacobi and the multigrid preconditioner, over whole
steps; the direct mode's launch count grows with the kernels it issues."""
import numpy as np
import pytest

from helpers import load_state, make_pair, opts, random_state

pytestmark = pytest.mark.gpu

INFLOW = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("precon", ["Diagonal", "PFMG"])
def test_direct_launches_match_graphs(built, precision, precon):
    n = 96
    pairs = [make_pair(n, n, source=INFLOW, body=(0.0, -2.0), precision=precision) for _ in range(2)]
    st = random_state(pairs[0][0], np.random.default_rng(12), scale=0.3, smooth=True)
    for o, c in pairs:
        load_state(o, c, st)
    ca, cb = pairs[0][1], pairs[1][1]
    cb.set_graphs(False)
    dt = 0.5 / n / 3.0
    so = opts(tol=1e-9, max_iter=5000, precon=precon)
    for k in range(3):
        sa = ca.step(dt, 3, so, raise_on_maxit=True)
        l0 = cb.launches
        sb = cb.step(dt, 3, so, raise_on_maxit=True)
        assert cb.launches - l0 > sb["iterations"]
        assert sa["iterations"] == sb["iterations"] and sa["div_l2"] == sb["div_l2"], k
        for f in ("q", "u", "v", "p"):
            assert np.array_equal(ca.download(f), cb.download(f)), (k, f)
