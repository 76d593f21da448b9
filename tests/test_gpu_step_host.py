"""cf_step_host (host buffers in and out, one call per step) gives the same
bits as cf_upload + cf_step + cf_download, in FP64 and mixed precision, with
both preconditioners."""
import numpy as np
import pytest

from cajitafluids_gb300.api import PinnedArray
from helpers import make_pair, opts, random_state

pytestmark = pytest.mark.gpu

INFLOW = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)


@pytest.mark.parametrize("precision,precon,periodic", [("fp64", "Diagonal", (False, False)),
                                                        ("fp64", "PFMG", (True, True)),
                                                        ("mixed", "PFMG", (False, False)),
                                                        ("mixed", "Diagonal", (True, False))])
def test_step_host_matches_separate_calls(built, precision, precon, periodic):
    n = 64
    rng = np.random.default_rng(3)
    o, a = make_pair(n, n, periodic=periodic, source=INFLOW, precision=precision)
    b = make_pair(n, n, periodic=periodic, source=INFLOW, precision=precision)[1]
    st = random_state(o, rng, scale=0.2)
    dt = 0.5 / n / 3.0
    so = opts(tol=1e-9, precon=precon)
    q, u, v = st["q"], st["u"], st["v"]
    hq, hu, hv = (PinnedArray(a.owned_shape(f)) for f in ("q", "u", "v"))
    hq.array[:], hu.array[:], hv.array[:] = q, u, v
    for k in range(3):
        # separate calls on context a
        a.upload("q", q)
        a.upload("u", u)
        a.upload("v", v)
        sa = a.step(dt, 3, so)
        q, u, v = a.download("q"), a.download("u"), a.download("v")
        # one call on context b, in place in page-locked buffers
        sb = b.step_host(dt, 3, so, hq.array, hu.array, hv.array, hq.array, hu.array, hv.array)
        assert sa["iterations"] == sb["iterations"] and sa["div_l2"] == sb["div_l2"], k
        for x, y in ((q, hq.array), (u, hu.array), (v, hv.array)):
            assert np.array_equal(x, y), k
    for h in (hq, hu, hv):
        h.free()


def test_step_host_outputs_optional_and_shapes_checked(built):
    o, c = make_pair(32, 32)
    st = random_state(o, np.random.default_rng(1))
    qo = np.empty(c.owned_shape("q"))
    c.step_host(0.001, 3, opts(), st["q"], st["u"], st["v"], q_out=qo)
    assert np.array_equal(qo, c.download("q"))
    with pytest.raises(ValueError):
        c.step_host(0.001, 3, opts(), st["q"], st["v"], st["u"])


def test_step_host_failed_setup_is_retried(built):
    """A first cf_step_host whose lazy set-up fails (an out-of-memory
    cudaMalloc, injected on the host) returns CF_ERR_NOMEM and leaves no
    half-made state: the next call creates what is missing and matches a
    context that never failed, bit for bit."""
    from cajitafluids_gb300 import _lib as L
    from cajitafluids_gb300.api import CfError
    lib = L.load()
    rng = np.random.default_rng(5)
    o, a = make_pair(48, 48, source=INFLOW, precision="mixed")
    b = make_pair(48, 48, source=INFLOW, precision="mixed")[1]
    st = random_state(o, rng, scale=0.2)
    dt = 0.5 / 48 / 3.0
    so = opts(tol=1e-9, precon="PFMG")
    outs_a = [np.empty(a.owned_shape(f)) for f in ("q", "u", "v")]
    outs_b = [np.empty(b.owned_shape(f)) for f in ("q", "u", "v")]
    # the mixed context's first cf_step_host allocates its staging buffers;
    # the first of them fails
    lib.cf_test_fail_alloc(1)
    try:
        with pytest.raises(CfError) as e:
            a.step_host(dt, 3, so, st["q"], st["u"], st["v"], *outs_a)
        assert e.value.code == L.CF_ERR_NOMEM
    finally:
        lib.cf_test_fail_alloc(0)
    sa = a.step_host(dt, 3, so, st["q"], st["u"], st["v"], *outs_a)
    sb = b.step_host(dt, 3, so, st["q"], st["u"], st["v"], *outs_b)
    assert sa["iterations"] == sb["iterations"]
    for x, y in zip(outs_a, outs_b):
        assert np.array_equal(x, y)
