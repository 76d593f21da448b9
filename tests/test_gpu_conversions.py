"""The integer-pipe FP64 <-> FP32 conversions used by the mixed-precision
kernels (the double-float pairs of u, v and b, the double-float pressure to
FP64) give the hardware's results bit for bit:
round to nearest even, exact widening, zeros, subnormals, infinities, NaN,
the overflow threshold and exact ties."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_conversions_match_ieee(built):
    from cajitafluids_gb300 import Context
    rng = np.random.default_rng(5)
    vals = [rng.standard_normal(50000) * 10.0 ** rng.integers(-45, 45, 50000)]
    f = rng.standard_normal(20000).astype(np.float32)
    ulp = np.spacing(f).astype(np.float64)
    d = f.astype(np.float64)
    vals += [d + ulp / 2, d - ulp / 2, d + ulp * 0.4999999, d - ulp * 0.5000001]  # ties and near-ties
    fmax = float(np.finfo(np.float32).max)
    vals.append(np.array([0.0, -0.0, 1.0, -1.0, fmax, -fmax, fmax * (1 + 2.0 ** -25), fmax * (1 + 2.0 ** -23),
                          1.1754943508222875e-38, 1.17549e-38, 1e-40, -3e-45, 1e-50, 1e300, -1e300, np.inf, -np.inf,
                          np.nan]))
    d = np.concatenate(vals)
    c = Context(8, 8)
    got_f, got_w = c.test_conversions(d)
    with np.errstate(over="ignore"):
        want_f = d.astype(np.float32)
    nan = np.isnan(want_f)  # NaN payloads are not compared
    assert np.array_equal(np.isnan(got_f), nan) and np.isnan(got_w[nan]).all()
    assert np.array_equal(got_f[~nan].view(np.uint32), want_f[~nan].view(np.uint32))
    want_w = want_f[~nan].astype(np.float64)
    assert np.array_equal(got_w[~nan].view(np.uint64), want_w.view(np.uint64))
