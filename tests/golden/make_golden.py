"""Generates the golden fixtures in this directory.

    python tests/golden/make_golden.py

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


def main():
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
