"""Seeded synthetic workloads for the benchmark configurations.

The reference has no public dataset; every input here is generated from a
seed.  Velocities come from a streamfunction psi sampled on the nodes, so
u = d(psi)/dy and v = -d(psi)/dx taken as node differences give a MAC field
whose discrete divergence is zero up to round-off.

  smoke / config 0 : 256^2 walls, zero state, inflow block (x in [.45,.55],
                     y in [.10,.15], q = 1, v = 3), linear, dt = 0.5 dx / 3
  config 1         : 1024^2 walls, cubic, config-0 inflow, buoyancy (0, -9.8)
                     scaled by the advected quantity (extension)
  config 2         : 4096^2 periodic, spectral velocity (per-mode velocity
                     power ~ k^-11/3, k <= 64, rms |u| = 1) and spectral
                     scalar (per-mode power ~ k^-3, mapped to [0, 1]),
                     dt = 0.5 dx / max |u|
  config 3         : 512^2 walls, wall-windowed spectral velocity, 8 Gaussian
                     blobs (sigma 0.03) as scalar
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional, Tuple

import numpy as np

SOLID, FREE = 0, 1


@dataclass
class Workload:
    name: str
    nx: int
    ny: int
    periodic: Tuple[bool, bool] = (False, False)
    bc: Tuple[int, int, int, int] = (SOLID, SOLID, SOLID, SOLID)
    source: Optional[tuple] = None          # (location, size, velocity, quantity)
    source_mode: int = 0
    body: Tuple[float, float] = (0.0, 0.0)
    body_density_scaled: bool = False
    density: float = 0.1                    # reference CLI default (examples/advection.cpp:181)
    dt: float = 0.0
    order: int = 3
    tol: float = 1e-8
    abs_tol: float = 0.0
    max_iter: int = 100000
    precon: str = "Diagonal"                # PCG preconditioner name (PFMG/SMG/MG: multigrid)
    steps: int = 1
    q0: Optional[np.ndarray] = None
    u0: Optional[np.ndarray] = None
    v0: Optional[np.ndarray] = None
    extra: dict = field(default_factory=dict)


def _spectral_field(n_nodes_x, n_nodes_y, n_period, slope, kmax, rng):
    """Real periodic field on an n_period^2 grid with per-mode power |k|^slope
    for 1 <= |k| <= kmax and Gaussian random coefficients, returned on the
    first n_nodes_y x n_nodes_x points (periodic extension)."""
    n = n_period
    kx = np.fft.rfftfreq(n, 1.0 / n)
    ky = np.fft.fftfreq(n, 1.0 / n)
    # only a (2 kmax + 1) x (kmax + 1) block of modes is non-zero
    ky_sel = np.concatenate([np.arange(0, kmax + 1), np.arange(n - kmax, n)]) if n > 2 * kmax + 1 else np.arange(n)
    kx_sel = np.arange(0, min(kmax + 1, kx.size))
    KY, KX = np.meshgrid(ky[ky_sel], kx[kx_sel], indexing="ij")
    k = np.sqrt(KX ** 2 + KY ** 2)
    amp = np.zeros_like(k)
    m = (k >= 1.0) & (k <= kmax)
    amp[m] = k[m] ** (slope / 2.0)
    coef = (rng.standard_normal(k.shape) + 1j * rng.standard_normal(k.shape)) * amp
    spec = np.zeros((n, n // 2 + 1), dtype=np.complex128)
    spec[np.ix_(ky_sel, kx_sel)] = coef
    f = np.fft.irfft2(spec, s=(n, n))
    # periodic extension to the requested node count
    iy = np.arange(n_nodes_y) % n
    ix = np.arange(n_nodes_x) % n
    return f[np.ix_(iy, ix)]


def mac_from_streamfunction(psi: np.ndarray, dx: float, periodic: bool):
    """u on I-faces, v on J-faces from node values psi[j, i].

    periodic: psi is (n, n) and indices wrap; walls: psi is (n+1, n+1)."""
    if periodic:
        psi_e = np.concatenate([psi, psi[:1]], axis=0)
        psi_e = np.concatenate([psi_e, psi_e[:, :1]], axis=1)
        u = (psi_e[1:, :-1] - psi_e[:-1, :-1]) / dx      # (n, n): I-faces i = 0..n-1
        v = -(psi_e[:-1, 1:] - psi_e[:-1, :-1]) / dx     # (n, n): J-faces j = 0..n-1
    else:
        u = (psi[1:, :] - psi[:-1, :]) / dx              # (n, n+1)
        v = -(psi[:, 1:] - psi[:, :-1]) / dx             # (n+1, n)
    return u, v


def spectral_velocity(n: int, seed: int, periodic: bool, kmax: int = 64):
    rng = np.random.default_rng(seed)
    dx = 1.0 / n
    slope = -11.0 / 3.0 - 2.0   # psi power = velocity power / k^2
    if periodic:
        psi = _spectral_field(n, n, n, slope, kmax, rng)
    else:
        psi = _spectral_field(n + 1, n + 1, n, slope, kmax, rng)
        x = np.arange(n + 1) * dx
        w = np.sin(np.pi * x)
        psi = psi * w[None, :] * w[:, None]
        psi[0, :] = psi[-1, :] = 0.0
        psi[:, 0] = psi[:, -1] = 0.0
    u, v = mac_from_streamfunction(psi, dx, periodic)
    rms = np.sqrt(np.mean(u * u) + np.mean(v * v))
    return u / rms, v / rms


def spectral_scalar(n: int, seed: int, kmax: int = 64):
    rng = np.random.default_rng(seed)
    f = _spectral_field(n, n, n, -3.0, kmax, rng)
    lo, hi = f.min(), f.max()
    return (f - lo) / (hi - lo)


def gaussian_blobs(n: int, seed: int, count: int = 8, sigma: float = 0.03):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.15, 0.85, size=(count, 2))
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="xy")
    q = np.zeros((n, n))
    for cx, cy in c:
        q += np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * sigma * sigma))
    return q


def config0(n: int = 256, steps: int = 100) -> Workload:
    dx = 1.0 / n
    return Workload("config0-walls-inflow-linear", n, n,
                    source=((0.45, 0.10), (0.10, 0.05), (0.0, 3.0), 1.0),
                    dt=0.5 * dx / 3.0, order=1, tol=1e-8, steps=steps,
                    q0=np.zeros((n, n)), u0=np.zeros((n, n + 1)), v0=np.zeros((n + 1, n)))


def config1(n: int = 1024, steps: int = 500) -> Workload:
    w = config0(n, steps)
    w.name = "config1-walls-inflow-cubic-buoyancy"
    w.order = 3
    w.tol = 1e-10
    w.body = (0.0, -9.8)
    w.body_density_scaled = True
    return w


def config2(n: int = 4096, steps: int = 200, seed: int = 2) -> Workload:
    u, v = spectral_velocity(n, seed, periodic=True)
    q = spectral_scalar(n, seed + 1000)
    dx = 1.0 / n
    umax = max(np.abs(u).max(), np.abs(v).max())
    return Workload("config2-periodic-spectral", n, n, periodic=(True, True), dt=0.5 * dx / umax,
                    order=3, tol=0.0, abs_tol=1e-8, steps=steps, q0=q, u0=u, v0=v)


def config3(n: int = 512, steps: int = 200, seed: int = 3) -> Workload:
    u, v = spectral_velocity(n, seed, periodic=False)
    q = gaussian_blobs(n, seed + 1)
    dx = 1.0 / n
    umax = max(np.abs(u).max(), np.abs(v).max())
    w = Workload("config3-walls-blobs", n, n, dt=0.5 * dx / umax, order=3, tol=1e-10, steps=steps,
                 q0=q, u0=u, v0=v)
    w.extra["target"] = gaussian_blobs(n, seed + 2)
    return w


def config4(n: int = 8192, steps: int = 100, seed: int = 4) -> Workload:
    """Large mixed forward + adjoint: walls, cubic values, seeded spectral
    velocity (no normal flow at the walls) and scalar as in config 2,
    projection to ||div u||_L2 <= 1e-8; loss 1/2 |q(T) - target|^2 with a
    second seeded spectral scalar as the target."""
    u, v = spectral_velocity(n, seed, periodic=False)
    q = spectral_scalar(n, seed + 1000)
    dx = 1.0 / n
    umax = max(np.abs(u).max(), np.abs(v).max())
    w = Workload("config4-walls-spectral-mixed-adjoint", n, n, dt=0.5 * dx / umax, order=3, tol=0.0,
                 abs_tol=1e-8, steps=steps, q0=q, u0=u, v0=v)
    w.extra["target"] = spectral_scalar(n, seed + 2000)
    return w
