"""Seeded synthetic point geometries and wavenumbers for the far-field workloads.

These stand in for the BEAST meshes / RWG basis-function positions the
reference clusters (``evaluation/singleblock.jl:213-226``,
``evaluation/benchmarking.jl``): points on surfaces with a fixed density of
about 100 points per wavelength squared.
"""
from __future__ import annotations

import math

import numpy as np

GOLDEN_ANGLE = math.pi * (3.0 - math.sqrt(5.0))


def plane_pair(n: int, seed: int, z_obs: float = 4.0):
    """Two iid-uniform point sets on [0,1]^2 at z=0 (sources) and z=z_obs (observers).

    Draw order: sources first, then observers, from ``numpy.random.default_rng(seed)``.
    """
    rng = np.random.default_rng(seed)
    src = np.zeros((n, 3))
    obs = np.zeros((n, 3))
    src[:, :2] = rng.random((n, 2))
    obs[:, :2] = rng.random((n, 2))
    obs[:, 2] = z_obs
    return obs, src


def fibonacci_sphere(n: int, axes=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Fibonacci lattice on the unit sphere, optionally stretched to an ellipsoid."""
    i = np.arange(n, dtype=np.float64)
    z = 1.0 - (2.0 * i + 1.0) / n
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = i * GOLDEN_ANGLE
    pts = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    return pts * np.asarray(axes, dtype=np.float64)[None, :]


def cube_surface(n: int, seed: int, half: float = 1.0) -> np.ndarray:
    """iid-uniform points on the six faces of the cube [-half, half]^3 (equal share per face)."""
    rng = np.random.default_rng(seed)
    face = np.arange(n) % 6
    uv = rng.uniform(-half, half, size=(n, 2))
    pts = np.empty((n, 3))
    ax = face // 2
    sgn = np.where(face % 2 == 0, -half, half)
    for a in range(3):
        m = ax == a
        others = [b for b in range(3) if b != a]
        pts[m, a] = sgn[m]
        pts[m, others[0]] = uv[m, 0]
        pts[m, others[1]] = uv[m, 1]
    return pts


def ellipsoid_area(a: float, b: float, c: float) -> float:
    """Thomsen's approximation of the ellipsoid surface area (|rel. err| < 1.1 %)."""
    p = 1.6075
    return 4.0 * math.pi * (((a * b) ** p + (a * c) ** p + (b * c) ** p) / 3.0) ** (1.0 / p)


def wavenumber(n_points: int, area: float, points_per_lambda2: float = 100.0) -> float:
    """k = 2 pi / lambda with lambda chosen so there are ``points_per_lambda2`` points per lambda^2."""
    lam = math.sqrt(points_per_lambda2 * area / n_points)
    return 2.0 * math.pi / lam


def shape_points(shape: str, n: int, seed: int):
    """(points, area) for 'sphere', 'ellipsoid' (1, 0.5, 0.25) or 'cube' (edge 2)."""
    if shape == "sphere":
        return fibonacci_sphere(n), 4.0 * math.pi
    if shape == "ellipsoid":
        return fibonacci_sphere(n, (1.0, 0.5, 0.25)), ellipsoid_area(1.0, 0.5, 0.25)
    if shape == "cube":
        return cube_surface(n, seed), 24.0
    raise ValueError(f"unknown shape {shape!r}")


def complex_gaussian(n: int, seed: int, nrhs: int | None = None) -> np.ndarray:
    """RHS with Re and Im iid N(0,1), from ``default_rng(seed)``; shape (n,) or (n, nrhs) column-major."""
    rng = np.random.default_rng(seed)
    if nrhs is None:
        return rng.standard_normal(n) + 1j * rng.standard_normal(n)
    x = rng.standard_normal((nrhs, n)) + 1j * rng.standard_normal((nrhs, n))
    return np.asfortranarray(x.T)


def plane_waves(points: np.ndarray, k: float, n_dirs: int, seed: int) -> np.ndarray:
    """Columns exp(-i k d.x) for directions d uniform on S^2 (seeded); (n, n_dirs) column-major."""
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((n_dirs, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.asfortranarray(np.exp(-1j * k * (points @ d.T)))
