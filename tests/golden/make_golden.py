"""Generates the golden fixtures in this directory from the CPU oracle.

    python tests/golden/make_golden.py

The reference (Kokkos + Cabana/Cajita + HYPRE + MPI) cannot be built or
imported here, so the fixtures are oracle outputs: they pin the oracle
against regressions and give the GPU path fixed expected values
(tests/test_golden.py, bit for bit).
Every input is generated from a seed below.
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


def main():
    np.savez_compressed(os.path.join(HERE, "config0_32.npz"), **config0_small())
    np.savez_compressed(os.path.join(HERE, "periodic_spectral_32.npz"), **periodic_small())
    np.savez_compressed(os.path.join(HERE, "interp_kat_24.npz"), **interpolation_kat())
    np.savez_compressed(os.path.join(HERE, "walls_buoyancy_mg_48.npz"), **walls_buoyancy_mg())
    print("wrote", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))


if __name__ == "__main__":
    main()
