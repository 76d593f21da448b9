"""Shared set-up for parity tests: one spec drives both the oracle and the GPU."""
from __future__ import annotations

import numpy as np

from cajitafluids_gb300 import Context, SolverOptions
from cajitafluids_gb300.workloads import mac_from_streamfunction

FIELDS = ("q", "u", "v")


def make_pair(nx, ny, periodic=(False, False), bc=(0, 0, 0, 0), source=None, source_mode=0, body=(0.0, 0.0),
              body_density_scaled=False, density=0.1, quirks=0, precision="fp64", lo=(0.0, 0.0), hi=None,
              precon_none=False, precon_mg=False, warm_start=False):
    from oracle import Oracle
    if hi is None:
        hi = (lo[0] + 1.0, lo[1] + ny / nx)
    o = Oracle(nx, ny, lo=lo, hi=hi, periodic=periodic, bc=bc, source=source, source_mode=source_mode, body=body,
               body_density_scaled=body_density_scaled, density=density, quirks=quirks, precon_none=precon_none,
               precon_mg=precon_mg, warm_start=warm_start)
    c = Context(nx, ny, lo=lo, hi=hi, periodic=periodic, precision=precision)
    c.set_bc(bc)
    if source is not None:
        c.set_source(source[0], source[1], source[2], source[3], source_mode)
    c.set_body_force(body, body_density_scaled)
    c.set_density(density)
    c.set_quirks(quirks)
    if warm_start:
        c.set_warm_start(True)
    return o, c


def random_state(o, rng, scale=1.0, smooth=False):
    """Random q, u, v of the oracle's owned shapes (optionally divergence-free)."""
    out = {}
    ny, nx = o.shape("q")
    if smooth:
        periodic = o.shape("u")[1] == nx
        n_nodes = (ny, nx) if periodic else (ny + 1, nx + 1)
        psi = rng.standard_normal(n_nodes) * 0.01
        if not periodic:
            psi[0, :] = psi[-1, :] = psi[:, 0] = psi[:, -1] = 0.0
        u, v = mac_from_streamfunction(psi, 1.0 / nx, periodic) if nx == ny else (None, None)
        if u is None:
            u = rng.standard_normal(o.shape("u")) * scale
            v = rng.standard_normal(o.shape("v")) * scale
        out["u"], out["v"] = u * scale, v * scale
    else:
        out["u"] = rng.standard_normal(o.shape("u")) * scale
        out["v"] = rng.standard_normal(o.shape("v")) * scale
    out["q"] = rng.uniform(0.0, 1.0, o.shape("q"))
    # wall-normal velocities are zero, as _addInputs leaves them before every
    # projection; otherwise the all-Neumann pressure system is inconsistent
    ny, nx = o.shape("q")
    if out["u"].shape[1] == nx + 1:
        out["u"][:, 0] = 0.0
        out["u"][:, -1] = 0.0
    if out["v"].shape[0] == ny + 1:
        out["v"][0, :] = 0.0
        out["v"][-1, :] = 0.0
    return out


def load_state(o, c, state):
    for f in FIELDS:
        o.set(f, state[f])
        c.upload(f, state[f])


def assert_fields_equal(o, c, fields=FIELDS, tag=""):
    for f in fields:
        a = o.get(f)
        b = c.download(f)
        if not np.array_equal(a, b):
            d = np.abs(a - b)
            k = np.unravel_index(np.argmax(d), d.shape)
            raise AssertionError(f"{tag} field {f}: {np.count_nonzero(a != b)} of {a.size} differ, "
                                 f"max |diff| {d.max():.3e} at {k} (oracle {a[k]!r}, gpu {b[k]!r})")


def opts(tol=1e-8, max_iter=20000, abs_tol=0.0, **kw):
    return SolverOptions(tol=tol, abs_tol=abs_tol, max_iter=max_iter, **kw)


def pair_round(a):
    """FP64 values as a mixed context stores velocities: the double-float pair
    hi = fl32(a), lo = fl32(a - hi), read back as hi + lo (about 48 bits)."""
    a = np.asarray(a, dtype=np.float64)
    hi = a.astype(np.float32).astype(np.float64)
    lo = (a - hi).astype(np.float32).astype(np.float64)
    return hi + lo

