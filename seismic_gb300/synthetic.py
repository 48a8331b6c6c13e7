"""Seeded synthetic velocity models (stand-ins for the OpenFWI / Kaggle data).

The competition data the reference was tuned on is not available here, so the
workloads use seeded models with its shapes (70x70 and larger grids, 1500-4500
m/s) and the three families named for the benchmark: layered, faulted and
curved.  Every generator takes a ``numpy.random.Generator`` so that runs are
reproducible from a recorded seed.
"""
from __future__ import annotations

import numpy as np
from scipy.ndimage import gaussian_filter

VMIN, VMAX = 1500.0, 4500.0


def _layer_velocities(rng, n):
    return np.sort(rng.uniform(VMIN, VMAX, n))


def _interfaces(rng, nz, n):
    # up to n-1 interface depths strictly inside the model, sorted (fewer on tiny grids)
    cand = np.arange(3, nz - 2) if nz >= 8 else np.arange(1, max(nz, 2))
    return np.sort(rng.choice(cand, size=min(n - 1, len(cand)), replace=False))


def layered(rng: np.random.Generator, nz: int = 70, nx: int = 70) -> np.ndarray:
    """3-5 horizontal layers, velocities uniform in [1500, 4500] sorted increasing with depth."""
    n = int(rng.integers(3, 6))
    vel = _layer_velocities(rng, n)
    depth = _interfaces(rng, nz, n)
    z = np.arange(nz)[:, None]
    layer = np.searchsorted(depth, z, side="right")
    return np.broadcast_to(vel[layer], (nz, nx)).astype(np.float64).copy()


def faulted(rng: np.random.Generator, nz: int = 70, nx: int = 70) -> np.ndarray:
    """A layered model offset by 5-20 cells across a random dipping line."""
    n = int(rng.integers(3, 6))
    vel = _layer_velocities(rng, n)
    depth = _interfaces(rng, nz, n)
    throw = int(rng.integers(5, 21))
    x0 = rng.uniform(0.2 * nx, 0.8 * nx)
    dip = np.tan(np.deg2rad(rng.uniform(-60, 60)))
    z = np.arange(nz)[:, None].astype(np.float64)
    x = np.arange(nx)[None, :].astype(np.float64)
    hanging = x > x0 + dip * (z - nz / 2)
    zz = np.where(hanging, z - throw, z)
    layer = np.searchsorted(depth, zz, side="right")
    return vel[np.clip(layer, 0, n - 1)].astype(np.float64)


def curved(rng: np.random.Generator, nz: int = 70, nx: int = 70) -> np.ndarray:
    """Layers with sinusoidal interfaces of amplitude 3-10 cells."""
    n = int(rng.integers(3, 6))
    vel = _layer_velocities(rng, n)
    depth = _interfaces(rng, nz, n).astype(np.float64)
    amp = rng.uniform(3, 10)
    k = rng.uniform(0.5, 2.5) * 2 * np.pi / nx
    ph = rng.uniform(0, 2 * np.pi)
    x = np.arange(nx)[None, :]
    z = np.arange(nz)[:, None].astype(np.float64)
    shift = amp * np.sin(k * x + ph)
    layer = np.zeros((nz, nx), dtype=np.int64)
    for d in depth:
        layer += (z >= d + shift).astype(np.int64)
    return vel[np.clip(layer, 0, n - 1)].astype(np.float64)


FAMILIES = {"layered": layered, "faulted": faulted, "curved": curved}


def model(rng: np.random.Generator, family: str, nz: int = 70, nx: int = 70) -> np.ndarray:
    return FAMILIES[family](rng, nz, nx)


def perturbed(rng: np.random.Generator, v: np.ndarray, rel: float = 0.05, sigma: float = 3.0) -> np.ndarray:
    """Copy with a +-rel Gaussian-smoothed multiplicative perturbation (true model for targets)."""
    noise = gaussian_filter(rng.normal(0.0, 1.0, v.shape), sigma, mode="nearest")
    noise /= max(np.abs(noise).max(), 1e-12)
    return v * (1.0 + rel * noise)


def smoothed(v: np.ndarray, sigma_cells: float) -> np.ndarray:
    """Gaussian-smoothed start model."""
    return gaussian_filter(v, sigma_cells, mode="nearest")


def to_vector(v: np.ndarray, min_vel: float | None = None) -> np.ndarray:
    """Reference model-vector layout: row-major velocities then min_vel
    (core/kaggle_support.py:243-245); min_vel defaults to min(v)."""
    mv = float(v.min()) if min_vel is None else float(min_vel)
    return np.concatenate([np.asarray(v, np.float64).ravel(), [mv]])


def batch(seed: int, n: int, nz: int = 70, nx: int = 70, families=("layered", "faulted", "curved")):
    """n model vectors cycling through the families, plus target vectors from
    perturbed copies; returns (vecs (n, nz*nx+1), true_vecs (n, nz*nx+1), family names)."""
    rng = np.random.default_rng(seed)
    vecs, trues, fams = [], [], []
    for i in range(n):
        fam = families[i % len(families)]
        v = model(rng, fam, nz, nx)
        vt = perturbed(rng, v)
        vecs.append(to_vector(v))
        trues.append(to_vector(vt))
        fams.append(fam)
    return np.stack(vecs), np.stack(trues), fams
