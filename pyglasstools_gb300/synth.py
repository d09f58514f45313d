"""Seeded synthetic polydisperse frames of the shapes used for measurement.

Recipe (per frame):
  * diameters d ~ P(sigma) ~ sigma^-3 on [0.73, 1.62], by inverse CDF
    sigma = (smin^-2 - u (smin^-2 - smax^-2))^(-1/2);
  * number density 1: box edge L = N^(1/dim), box centred at the origin;
  * a square (cubic) lattice of ceil(N^(1/dim)) sites per side with spacing
    L / sites, a seeded subset of N sites, Gaussian jitter (std 0.08), wrapped;
  * velocities Maxwell-Boltzmann at temperature T with m = 1, mean removed.
numpy's PCG64 generator makes the frames identical on every platform.
"""
from __future__ import annotations

import math

import numpy as np

SIGMA_MIN, SIGMA_MAX = 0.73, 1.62


class SynthFrame:
    def __init__(self, dim, L, pos, vel, mass, diam):
        self.dim = dim
        self.L = L
        self.pos = pos
        self.vel = vel
        self.mass = mass
        self.diam = diam

    @property
    def N(self):
        return len(self.pos)


def make_frame(N: int, dim: int = 2, seed: int = 0, T: float | None = None,
               jitter: float = 0.08) -> SynthFrame:
    if T is None:
        T = 0.3 if dim == 2 else 0.5
    rng = np.random.default_rng(seed)
    L = float(N) ** (1.0 / dim)
    sites = int(math.ceil(N ** (1.0 / dim) - 1e-9))
    while sites ** dim < N:
        sites += 1
    a = L / sites
    pick = np.sort(rng.choice(sites ** dim, size=N, replace=False))
    coords = np.stack(np.unravel_index(pick, (sites,) * dim), axis=1).astype(np.float64)
    pos = np.zeros((N, 3))
    pos[:, :dim] = -0.5 * L + (coords + 0.5) * a + rng.normal(0.0, jitter, size=(N, dim))
    pos[:, :dim] -= L * np.floor((pos[:, :dim] + 0.5 * L) / L)  # wrap into [-L/2, L/2)
    u = rng.random(N)
    smin2, smax2 = SIGMA_MIN ** -2, SIGMA_MAX ** -2
    diam = (smin2 - u * (smin2 - smax2)) ** -0.5
    vel = np.zeros((N, 3))
    vel[:, :dim] = rng.normal(0.0, math.sqrt(T), size=(N, dim))
    vel[:, :dim] -= vel[:, :dim].mean(axis=0)
    mass = np.ones(N)
    return SynthFrame(dim, L, pos, vel, mass, diam)


def lattice_grid(L: float, nmax: int, dim: int = 2) -> np.ndarray:
    """The ikcalculator grid (irvingkirkwood/__init__.py:44-51): linspace(-L/2, L/2,
    nmax) per axis, both ends included, x outermost and the last axis innermost."""
    pts = np.linspace(-L / 2.0, +L / 2.0, nmax)
    if dim == 2:
        gx, gy = np.meshgrid(pts, pts, indexing="ij")
        return np.stack([gx.ravel(), gy.ravel(), np.zeros(gx.size)], axis=1)
    gx, gy, gz = np.meshgrid(pts, pts, pts, indexing="ij")
    return np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1)
