"""Generates the golden fixtures in this directory.

    python tests/golden/make_golden.py           # the small fixtures
    python tests/golden/make_golden.py --long    # also the full-length config 0 / config 1 runs

reference_*.npz come from the reference's own code: its src/*.hpp compiled
unchanged against the serial Kokkos/Cajita/MPI stand-ins in oracle/refshim
and run through createSolver("serial", ...) with the "Reference" solver
(oracle/reference.py).  They are written only where the reference's sources
are present; elsewhere the committed files are kept.  The other fixtures
are outputs of the CPU oracle, which equals the reference's code bit for
bit where both run (tests/test_reference_pin.py) and extends it to the
multigrid preconditioner, periodic axes and linear values.  All of them
give the GPU path fixed expected values (tests/test_golden.py, bit for
bit).  Every input is generated from a seed below.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import Oracle  # noqa: E402
from cajitafluids_gb300.workloads import spectral_scalar, spectral_velocity  # noqa: E402

INFLOW = ((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0)


def config0_small(n=32, steps=10):
    """Config-0 problem (walls, zero state, inflow, linear) at n^2."""
    dt = 0.5 * (1.0 / n) / 3.0
    o = Oracle(n, n, source=INFLOW, density=0.1)
    its, div = [], []
    s = o.setup(dt, tol=1e-8, max_iter=20000)
    its.append(s["iterations"])
    div.append(s["div_l2"])
    for _ in range(steps):
        s = o.step(dt, 1, tol=1e-8, max_iter=20000)
        its.append(s["iterations"])
        div.append(s["div_l2"])
    return dict(n=n, dt=dt, steps=steps, order=1, tol=1e-8, q=o.get("q"), u=o.get("u"), v=o.get("v"),
                p=o.get("p"), iterations=np.array(its), div_l2=np.array(div))


def periodic_small(n=32, steps=6, seed=5):
    """Periodic spectral problem (config-2 shape) at n^2, cubic, abs tol."""
    u, v = spectral_velocity(n, seed, True, kmax=6)
    q = spectral_scalar(n, seed + 1, kmax=6)
    dt = 0.5 / n / max(np.abs(u).max(), np.abs(v).max())
    o = Oracle(n, n, periodic=(True, True), density=0.1)
    o.set("q", q)
    o.set("u", u)
    o.set("v", v)
    its = []
    for _ in range(steps):
        s = o.step(dt, 3, tol=0.0, abs_tol=1e-10, max_iter=20000)
        its.append(s["iterations"])
    return dict(n=n, dt=dt, steps=steps, order=3, abs_tol=1e-10, q0=q, u0=u, v0=v, q=o.get("q"), u=o.get("u"),
                v=o.get("v"), p=o.get("p"), iterations=np.array(its))


def walls_buoyancy_mg(n=48, steps=6):
    """Walls, the config-0 inflow, gravity scaled by the quantity (extension
    Q5), cubic values, PCG + the multigrid preconditioner (the PFMG name),
    from a zero state."""
    dt = 0.5 * (1.0 / n) / 3.0
    o = Oracle(n, n, source=INFLOW, body=(0.0, -9.8), body_density_scaled=True, density=0.1, precon_mg=True)
    its, div = [], []
    s = o.setup(dt, tol=1e-10, max_iter=500)
    its.append(s["iterations"])
    div.append(s["div_l2"])
    for _ in range(steps):
        s = o.step(dt, 3, tol=1e-10, max_iter=500)
        its.append(s["iterations"])
        div.append(s["div_l2"])
    return dict(n=n, dt=dt, steps=steps, order=3, tol=1e-10, q=o.get("q"), u=o.get("u"), v=o.get("v"),
                p=o.get("p"), iterations=np.array(its), div_l2=np.array(div))


def interpolation_kat(n=24, seed=9):
    """Spline samples of seeded fields at seeded points, both orders."""
    rng = np.random.default_rng(seed)
    o = Oracle(n, n, periodic=(True, True))
    q = rng.standard_normal((n, n))
    u = rng.standard_normal((n, n))
    v = rng.standard_normal((n, n))
    o.set("q", q)
    o.set("u", u)
    o.set("v", v)
    o.fill_ghosts()
    xy = rng.uniform(0.0, 1.0, (200, 2))
    out = dict(n=n, q=q, u=u, v=v, xy=xy)
    for f in ("q", "u", "v"):
        for order in (1, 3):
            out[f"{f}_o{order}"] = o.sample(f, order, xy)
    out["trace"] = o.trace(xy, 0.01)
    return out


def reference_config0(n=64, steps=6):
    """The config-0 problem (walls, zero start, the inflow box, Q = 1,
    v = 3) run by the reference's own Solver<2>: setup + steps, cubic values
    and tol 1e-6 / 2000 iterations as the reference hard-codes them."""
    from oracle import reference as R
    dt = 0.5 * (1.0 / n) / 3.0
    prm = R.params(n, n, source=INFLOW, density=0.1, dt=dt)
    r = R.run(prm, steps=steps)
    return dict(n=n, dt=dt, steps=steps, density=0.1, q=r["q"], u=r["u"], v=r["v"], p=r["p"],
                iterations=r["iterations"])


def reference_random_walls_gravity(n=40, steps=4, seed=11):
    """A seeded random state, a FREE bottom wall, gravity and the inflow,
    run by the reference's own Solver<2>."""
    from oracle import reference as R
    rng = np.random.default_rng(seed)
    q0 = rng.uniform(0.0, 1.0, (n, n))
    u0 = rng.standard_normal((n, n + 1)) * 0.3
    v0 = rng.standard_normal((n + 1, n)) * 0.3
    dt = 0.25 / n
    bc = (0, 1, 0, 0)
    body = (0.0, -2.0)
    prm = R.params(n, n, bc=bc, source=INFLOW, body=body, density=0.1, dt=dt)
    r = R.run(prm, q0, u0, v0, steps=steps)
    return dict(n=n, dt=dt, steps=steps, density=0.1, bc=np.array(bc), body=np.array(body), q0=q0, u0=u0, v0=v0,
                q=r["q"], u=r["u"], v=r["v"], p=r["p"], iterations=r["iterations"])


def field_digest(arrays) -> str:
    """SHA-256 over the bytes of float64 arrays: equal digests mean equal
    bits, so a long run is compared bit for bit without storing its fields."""
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    return h.hexdigest()


def config0_full(steps=100):
    """Config 0 at its full size and length: 256^2, walls, zero start, the
    inflow box, linear values, Jacobi-PCG to 1e-8; setup + 100 steps.
    Stored as the iteration count and ||div u|| of every projection and a
    digest of the final q, u, v, p."""
    from cajitafluids_gb300.workloads import config0
    w = config0(steps=steps)
    o = Oracle(w.nx, w.ny, source=w.source, density=w.density)
    st = [o.setup(w.dt, tol=w.tol, max_iter=20000)]
    st += [o.step(w.dt, w.order, tol=w.tol, max_iter=20000) for _ in range(steps)]
    return dict(n=w.nx, steps=steps, dt=w.dt, tol=w.tol, order=w.order,
                iterations=np.array([x["iterations"] for x in st]), div_l2=np.array([x["div_l2"] for x in st]),
                div_linf=np.array([x["div_linf"] for x in st]),
                digest=field_digest([o.get(f) for f in ("q", "u", "v", "p")]), q_sum=float(o.get("q").sum()))


def config1_head(steps=2):
    """Config 1's problem (1024^2, walls, inflow, gravity scaled by the
    quantity, cubic values, Jacobi-PCG to 1e-10): setup + the first steps
    the oracle affords (about a minute per projection on 8 cores)."""
    from cajitafluids_gb300.workloads import config1
    w = config1(steps=steps)
    o = Oracle(w.nx, w.ny, source=w.source, body=w.body, body_density_scaled=w.body_density_scaled,
               density=w.density)
    st = [o.setup(w.dt, tol=w.tol, max_iter=50000)]
    st += [o.step(w.dt, w.order, tol=w.tol, max_iter=50000) for _ in range(steps)]
    return dict(n=w.nx, steps=steps, dt=w.dt, tol=w.tol, order=w.order,
                iterations=np.array([x["iterations"] for x in st]), div_l2=np.array([x["div_l2"] for x in st]),
                div_linf=np.array([x["div_linf"] for x in st]),
                digest=field_digest([o.get(f) for f in ("q", "u", "v", "p")]), q_sum=float(o.get("q").sum()))


def main():
    if "--long" in sys.argv:
        # full-length runs: several minutes of oracle time
        np.savez_compressed(os.path.join(HERE, "config0_256_full.npz"), **config0_full())
        np.savez_compressed(os.path.join(HERE, "config1_1024_head.npz"), **config1_head())
    from oracle import reference as R
    if R.available():
        np.savez_compressed(os.path.join(HERE, "reference_config0_64.npz"), **reference_config0())
        np.savez_compressed(os.path.join(HERE, "reference_random_walls_gravity_40.npz"),
                            **reference_random_walls_gravity())
    else:
        print("the reference's sources are not on this machine: reference_*.npz kept as committed")
    np.savez_compressed(os.path.join(HERE, "config0_32.npz"), **config0_small())
    np.savez_compressed(os.path.join(HERE, "periodic_spectral_32.npz"), **periodic_small())
    np.savez_compressed(os.path.join(HERE, "interp_kat_24.npz"), **interpolation_kat())
    np.savez_compressed(os.path.join(HERE, "walls_buoyancy_mg_48.npz"), **walls_buoyancy_mg())
    print("wrote", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))


if __name__ == "__main__":
    main()
