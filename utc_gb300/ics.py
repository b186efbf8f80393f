"""Seeded synthetic initial conditions for the nbody workloads.

All generators draw in float64 with numpy's PCG64 (``default_rng(seed)``)
and return float64 (n, 4) arrays -- positions (x, y, z, m) and velocities
(vx, vy, vz, w=1, the reference's unused fourth velocity component,
nbody.h:134) -- so the same draw can be cast to float32 for the kernels and
kept in float64 for the oracles.
"""
from __future__ import annotations

import math

import numpy as np


def uniform_cube(n, seed=0, half=1.0, vmax=0.01, mass_lo=0.5, mass_hi=1.5):
    """Positions U[-1,1]^3, velocities U[-0.01,0.01]^3, masses U[0.5,1.5]/n."""
    rng = np.random.default_rng(seed)
    pos = np.empty((n, 4), np.float64)
    vel = np.empty((n, 4), np.float64)
    pos[:, :3] = rng.uniform(-half, half, (n, 3))
    pos[:, 3] = rng.uniform(mass_lo, mass_hi, n) / n
    vel[:, :3] = rng.uniform(-vmax, vmax, (n, 3))
    vel[:, 3] = 1.0
    return pos, vel


def _isotropic(rng, r):
    """Random directions scaled by r, (len(r), 3)."""
    n = r.shape[0]
    cos_t = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * math.pi, n)
    sin_t = np.sqrt(1.0 - cos_t * cos_t)
    return np.stack([r * sin_t * np.cos(phi), r * sin_t * np.sin(phi), r * cos_t], axis=1)


def plummer(n, seed=0, a=1.0, G=1.0, M=1.0, rmax_frac=0.999, recenter=True):
    """Plummer sphere by the Aarseth, Henon & Wielen (1974) sampling.

    Radii from the inverted cumulative mass, r = a / sqrt(X^(-2/3) - 1) with
    X uniform in (0, rmax_frac]; speeds q * v_esc(r) with q drawn by
    rejection from g(q) = q^2 (1 - q^2)^(7/2) (the isotropic distribution
    function), v_esc = sqrt(2 G M / sqrt(r^2 + a^2)); isotropic directions.
    Equal masses M/n.  The centre of mass and its velocity are moved to 0.
    """
    rng = np.random.default_rng(seed)
    x1 = rng.uniform(0.0, rmax_frac, n)
    x1 = np.maximum(x1, 1e-300)
    r = a / np.sqrt(x1 ** (-2.0 / 3.0) - 1.0)
    pos = np.empty((n, 4), np.float64)
    pos[:, :3] = _isotropic(rng, r)
    pos[:, 3] = M / n
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        qq = rng.uniform(0.0, 1.0, todo.size)
        yy = rng.uniform(0.0, 0.1, todo.size)
        ok = yy < qq * qq * (1.0 - qq * qq) ** 3.5
        q[todo[ok]] = qq[ok]
        todo = todo[~ok]
    vesc = np.sqrt(2.0 * G * M) * (r * r + a * a) ** -0.25
    vel = np.empty((n, 4), np.float64)
    vel[:, :3] = _isotropic(rng, q * vesc)
    vel[:, 3] = 1.0
    if recenter:
        pos[:, :3] -= pos[:, :3].mean(axis=0)
        vel[:, :3] -= vel[:, :3].mean(axis=0)
    return pos, vel


def gaussian_targets(n, seed=1, sigma=0.5):
    """Target points y ~ N(0, sigma^2 I), (n, 3), for the trajectory loss."""
    rng = np.random.default_rng(seed)
    return rng.normal(0.0, sigma, (n, 3))


def batch_sizes(count=512, lo=128, hi=16384, seed=0):
    """System sizes drawn log-uniform in [lo, hi] (integers)."""
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi + 1), count))).astype(np.int64).clip(lo, hi)


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)
