"""Warm-started projections (extension; the reference cold-starts,
src/VelocityCorrector.hpp:272): each solve starts from the previous pressure.
FP64 stays bit-identical to the oracle's warm start; the warm start takes
fewer iterations than the cold one on a smoothly evolving flow."""
import numpy as np
import pytest

from cajitafluids_gb300 import CfError
from cajitafluids_gb300 import _lib as L
from helpers import assert_fields_equal, load_state, make_pair, opts, random_state

pytestmark = pytest.mark.gpu

INFLOW = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)


@pytest.mark.parametrize("precon", ["Diagonal", "PFMG"])
def test_warm_fp64_bitwise(built, precon):
    n = 64
    mg = precon == "PFMG"
    o, c = make_pair(n, n, source=INFLOW, density=0.1, precon_mg=mg, warm_start=True)
    oc, cc = make_pair(n, n, source=INFLOW, density=0.1, precon_mg=mg)
    dt = 0.5 * (1.0 / n) / 3.0
    kw = dict(tol=1e-9, max_iter=20000)
    o.setup(dt, **kw)
    c.setup(dt, opts(precon=precon, **kw))
    oc.setup(dt, **kw)
    cc.setup(dt, opts(precon=precon, **kw))
    warm_its, cold_its = [], []
    for k in range(8):
        so = o.step(dt, 3, **kw)
        sg = c.step(dt, 3, opts(precon=precon, **kw))
        assert so["iterations"] == sg["iterations"] and sg["status"] == 0, k
        warm_its.append(sg["iterations"])
        cold_its.append(cc.step(dt, 3, opts(precon=precon, **kw))["iterations"])
    assert_fields_equal(o, c, tag=f"warm {precon}")
    assert np.array_equal(o.get("p"), c.download("p"))
    assert sum(warm_its[2:]) < sum(cold_its[2:]), (warm_its, cold_its)


def test_warm_profiled_and_resident_agree(built):
    """The host-polled form (profiling on) and the device-resident graph give
    the same bits with a warm start."""
    res = []
    for prof in (False, True):
        o, c = make_pair(96, 64, periodic=(True, False), precon_mg=True, warm_start=True)
        load_state(o, c, random_state(o, np.random.default_rng(12)))
        c.profile_enable(prof)
        for _ in range(3):
            c.step(0.002, 3, opts(tol=1e-10, precon="PFMG"))
        res.append([c.download(f) for f in ("q", "u", "v", "p")])
    for a, b in zip(*res):
        assert np.array_equal(a, b)


def test_warm_mixed_mg(built):
    n = 128
    o, c = make_pair(n, n, source=INFLOW, density=0.1, precision="mixed", precon_mg=True, warm_start=True)
    cc = make_pair(n, n, source=INFLOW, density=0.1, precision="mixed", precon_mg=True)[1]
    dt = 0.5 * (1.0 / n) / 3.0
    o.setup(dt, tol=1e-9, max_iter=500)
    for ctx in (c, cc):
        ctx.setup(dt, opts(tol=1e-9, max_iter=500, precon="PFMG"))
    wi, ci = 0, 0
    for k in range(6):
        o.step(dt, 3, tol=1e-9, max_iter=500)
        sg = c.step(dt, 3, opts(tol=1e-9, max_iter=500, precon="PFMG"))
        assert sg["status"] == 0 and sg["r_norm"] <= 1e-9 * sg["b_norm"] * (1 + 1e-9)
        wi += sg["iterations"]
        ci += cc.step(dt, 3, opts(tol=1e-9, max_iter=500, precon="PFMG"))["iterations"]
    assert wi < ci
    for f in ("u", "v"):
        a, b = o.get(f), c.download(f)
        assert np.abs(a - b).max() <= 1e-4 * max(np.abs(a).max(), 1e-30), f


def test_warm_start_rejected_by_adjoint(built):
    from cajitafluids_gb300 import Context
    c = Context(32, 32)
    c.set_warm_start(True)
    with pytest.raises(CfError) as e:
        c.forward_checkpointed(2, 1, 0.001, 3)
    assert e.value.code == L.CF_ERR_UNSUPPORTED


def test_mixed_pressure_kept_as_pairs_then_warm(built):
    """A mixed projection without a warm start leaves its solution as
    double-float pairs (the gradient reads them; a download converts them).
    Switching the warm start on afterwards converts them first, so the next
    projection starts from the same FP64 pressure as in a context that kept
    the warm start on throughout: same pressure downloads, same second
    projection, bit for bit."""
    n = 96
    rng = np.random.default_rng(21)
    so = opts(tol=1e-9, max_iter=500, precon="PFMG")
    a = make_pair(n, n, periodic=(True, False), precision="mixed", precon_mg=True)
    b = make_pair(n, n, periodic=(True, False), precision="mixed", precon_mg=True, warm_start=True)
    st = random_state(a[0], rng, scale=0.1)
    for _, c in (a, b):
        load_state(a[0], c, st)
    ca, cb = a[1], b[1]
    ra = ca.project(0.002, so, raise_on_maxit=True)
    rb = cb.project(0.002, so, raise_on_maxit=True)
    assert ra["iterations"] == rb["iterations"]
    assert np.array_equal(ca.download("p"), cb.download("p"))
    ca.set_warm_start(True)
    for c in (ca, cb):
        for f in ("u", "v"):
            c.upload(f, st[f])
    ra = ca.project(0.002, so, raise_on_maxit=True)
    rb = cb.project(0.002, so, raise_on_maxit=True)
    assert ra["iterations"] == rb["iterations"]
    for f in ("u", "v", "p"):
        assert np.array_equal(ca.download(f), cb.download(f)), f
