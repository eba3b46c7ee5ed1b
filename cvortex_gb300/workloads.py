"""Seeded synthetic particle sets with the shapes and distributions of the
benchmark workloads (no public dataset is involved; all inputs are generated).

* uniform_cube: N particles, coordinates U[-1,1]^3, vorticity components
  N(0, 0.1^2), volume 8/N (the 10,000-particle plain workload, also the
  per-problem distribution of the batched and served workloads).
* vortex_ring: ring of radius 1; angle U[0, 2pi), radial and axial offsets
  N(0, 0.1^2) from the centreline; vorticity tangent to the ring with
  magnitude exp(-d^2 / (2 * 0.1^2)), d the offset distance; volume
  2 pi * 1 * pi * 0.1^2 / N (the 100,000-particle scale-up workload).
* gaussian_patch_2d: P2D particles with coordinates N(0, 0.5^2)^2,
  circulation exp(-|x|^2 / (2 * 0.5^2)) * A, area A = 2 pi 0.5^2 / N.
* cube_with_twins: uniform_cube where the last 1% of particles are replaced
  by twins of the first 1%, offset by |delta| ~ U(0, 1e-3 sigma) in a
  uniform direction (exercises rho << 1 pairs).
* wake_sheet: straight filament segments of length 0.02 tiling a 1 x 0.2
  sheet, strength N(0, 1).
* serve_stream: the served mixed-size request stream (Poisson arrivals; 60%
  P3D vel+dvort on uniform_cube, 25% P2D vel on gaussian_patch_2d, 15% F3D
  vel of a wake_sheet on as many tracer points in its box inflated by 0.1;
  sizes log-uniform on [500, 200,000]).
"""
from __future__ import annotations

import math

import numpy as np

from .abi import make_f3d, make_p2d, make_p3d

SEEDS = {"cube": 0, "ring": 1, "twins": 2, "batch": 3, "serve": 4, "patch": 5, "sheet": 6}


def uniform_cube(n: int, seed: int = SEEDS["cube"]):
    rng = np.random.Generator(np.random.PCG64(seed))
    coord = rng.uniform(-1.0, 1.0, (n, 3))
    vort = rng.normal(0.0, 0.1, (n, 3))
    return make_p3d(coord, vort, np.full(n, 8.0 / max(n, 1)))


def vortex_ring(n: int, seed: int = SEEDS["ring"], radius: float = 1.0, core: float = 0.1):
    rng = np.random.Generator(np.random.PCG64(seed))
    th = rng.uniform(0.0, 2.0 * math.pi, n)
    dr = rng.normal(0.0, core, n)
    dz = rng.normal(0.0, core, n)
    c, s = np.cos(th), np.sin(th)
    coord = np.stack([(radius + dr) * c, (radius + dr) * s, dz], axis=1)
    mag = np.exp(-(dr * dr + dz * dz) / (2.0 * core * core))
    vort = np.stack([-s * mag, c * mag, np.zeros(n)], axis=1)
    vol = 2.0 * math.pi * radius * math.pi * core * core / max(n, 1)
    return make_p3d(coord, vort, np.full(n, vol))


def gaussian_patch_2d(n: int, seed: int = SEEDS["patch"], width: float = 0.5):
    rng = np.random.Generator(np.random.PCG64(seed))
    coord = rng.normal(0.0, width, (n, 2))
    area = 2.0 * math.pi * width * width / max(n, 1)
    omega = np.exp(-(coord ** 2).sum(axis=1) / (2.0 * width * width))
    return make_p2d(coord, omega * area, np.full(n, area))


def cube_with_twins(n: int, sigma: float, frac: float = 0.01, seed: int = SEEDS["twins"]):
    p = uniform_cube(n, seed)
    rng = np.random.Generator(np.random.PCG64(seed + 1000))
    k = int(n * frac)
    if k:
        u = rng.normal(size=(k, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        mag = rng.uniform(0.0, 1e-3 * sigma, k)
        p["coord"][n - k:] = (p["coord"][:k].astype(np.float64) + u * mag[:, None]).astype(np.float32)
        p["vorticity"][n - k:] = uniform_cube(k, seed + 2000)["vorticity"]
    return p


def wake_sheet(n: int, seed: int = SEEDS["sheet"], seg: float = 0.02):
    """n straight segments of length `seg` laid span-wise on a 1 x 0.2 sheet."""
    rng = np.random.Generator(np.random.PCG64(seed))
    per_row = int(round(1.0 / seg))
    rows = max(1, -(-n // per_row))
    i = np.arange(n)
    x0 = (i % per_row) * seg - 0.5
    y = ((i // per_row) + 0.5) * (0.2 / rows) - 0.1
    start = np.stack([x0, y, np.zeros(n)], axis=1)
    end = np.stack([x0 + seg, y, np.zeros(n)], axis=1)
    return make_f3d(start, end, rng.normal(0.0, 1.0, n))


def sheet_targets(n: int, seed: int = SEEDS["sheet"] + 100):
    """Measurement points in the sheet's bounding box inflated by 0.1."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lo = np.array([-0.6, -0.2, -0.1])
    hi = np.array([0.6, 0.2, 0.1])
    return rng.uniform(lo, hi, (n, 3)).astype(np.float32)


def batch_sizes(count: int = 512, lo: int = 1000, hi: int = 50000, seed: int = SEEDS["batch"]):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.exp(rng.uniform(math.log(lo), math.log(hi), count)).astype(np.int64)


# ---- served request stream ---------------------------------------------------
SERVE_KINDS = ("p3d", "p2d", "f3d")
SERVE_MIX = (0.60, 0.25, 0.15)


def serve_stream(count: int, rate: float, lo: int = 500, hi: int = 200_000,
                 seed: int = SEEDS["serve"]):
    """Poisson arrivals at `rate` requests/s of a 60/25/15 mix of P3D vel+dvort,
    P2D vel and F3D vel requests, sizes log-uniform on [lo, hi].

    Returns (arrival_s, kinds, sizes, seeds); request i is built by
    serve_request_arrays(kinds[i], sizes[i], seeds[i]).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    gaps = rng.exponential(1.0 / rate, count)
    arrival = np.cumsum(gaps) - gaps[0]
    kinds = rng.choice(len(SERVE_KINDS), size=count, p=SERVE_MIX)
    sizes = np.exp(rng.uniform(math.log(lo), math.log(hi), count)).astype(np.int64)
    seeds = rng.integers(0, 2**31 - 1, count)
    return arrival, kinds, sizes, seeds


def serve_request_arrays(kind: int, n: int, seed: int):
    """Inputs of one served request: (particles or filaments, tracer points).

    P3D: uniform_cube; P2D: gaussian_patch_2d; F3D: wake_sheet filaments with
    n tracer points from sheet_targets."""
    n = int(n)
    if kind == 0:
        return uniform_cube(n, int(seed)), None
    if kind == 1:
        return gaussian_patch_2d(n, int(seed)), None
    return wake_sheet(n, int(seed)), sheet_targets(n, int(seed) + 1)
