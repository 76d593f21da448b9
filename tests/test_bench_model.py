"""The arithmetic behind bench.py's roofline line, checked without a GPU:
the multigrid level list it counts bytes over is the hierarchy the oracle
(and the library, whose FP64 V-cycle matches the oracle's bit for bit) builds,
and the minimal compulsory bytes per cell of one PCG iteration follow from the
per-stage word counts written in alg_bytes_per_iter's docstring."""
import numpy as np
import pytest

import bench
from oracle import Oracle


@pytest.mark.parametrize("nx,ny,periodic", [
    (64, 64, (True, True)), (96, 64, (False, False)), (200, 136, (True, False)),
    (2176, 1088, (False, False)), (33, 17, (False, False)), (48, 48, (True, True)),
])
def test_mg_levels_match_the_oracle_hierarchy(nx, ny, periodic):
    o = Oracle(nx, ny, hi=(nx / 64, ny / 64), periodic=periodic, precon_mg=True, bc=(1, 0, 0, 0))
    r = np.random.default_rng(3).standard_normal((ny, nx))
    _, nlev = o.mg_apply(1e-3, r)
    assert nlev == len(bench.mg_levels(nx, ny, periodic))


def _geometric(levels):
    n0 = levels[0][0] * levels[0][1]
    above = sum(a * c for a, c in levels[:-1]) / n0
    last = levels[-1][0] * levels[-1][1] / n0
    return above, last


def test_bytes_per_cell_4096_periodic():
    nx = ny = 4096
    lv = bench.mg_levels(nx, ny, (True, True))
    assert lv[-1] == (8, 8) and len(lv) == 10
    above, last = _geometric(lv)
    n = nx * ny
    per = lambda **k: bench.alg_bytes_per_iter(nx, ny, (True, True), **k) / n
    # mixed, an update after every iteration: K1 3 words, the x step fused with
    # the reliable update (R p 4, R x 8, R b 8, W x 8, W r 4 = 32), V-cycle 5.5
    # words per level cell, coarsest 2 words
    assert per(precon="PFMG", word=4, outer_frac=1.0, mixed=True) == pytest.approx(
        12 + 32 + 22 * above + 8 * last, rel=1e-12)
    assert per(precon="PFMG", word=4, outer_frac=1.0, mixed=True) == pytest.approx(73.333, abs=1e-3)
    # mixed, updates on half the iterations: the inner step also moves r (3 words + x pair)
    assert per(precon="PFMG", word=4, outer_frac=0.5, mixed=True) == pytest.approx(
        12 + 28 + 22 * above + 8 * last + 10, rel=1e-12)
    # FP64 MG: 3 + 5 words, r.z 2 words, V-cycle at 8 bytes
    assert per(precon="PFMG", word=8) == pytest.approx(24 + 40 + 16 + 44 * above + 16 * last, rel=1e-12)
    # Jacobi: 11 words per cell
    assert per(precon="Diagonal", word=4, mixed=True) == 44
    assert per(precon="Diagonal", word=8) == 88
