"""Seeded synthetic binary matrices with the shapes of the benchmark workloads.

The reference reports on SuiteSparse matrices that are not available here
(PARSEC/benzene, the astro-ph and cond-mat-2005 co-authorship graphs); these
generators produce stand-ins with the same dimensions, nonzero counts and
degree structure.  Every matrix goes through the reader's normalisation:
(row, col) pairs sorted and de-duplicated.

  uniform_matrix      3001 x 2048, 0.5 % i.i.d. positions          (small plain case)
  banded_powerlaw     8219^2 symmetric, power-law degrees, band     (benzene-shaped)
  uniform_powerlaw    16706^2 / 40421^2 symmetric, power-law degrees (graph-shaped)
  batch_matrices      64 matrices, log-uniform dims and densities   (batched case)
"""
from __future__ import annotations

import math

import numpy as np

from .sparse_fft import COOMatrix


def normalise(rows: int, cols: int, r: np.ndarray, c: np.ndarray) -> COOMatrix:
    """Sort by (row, col) and drop duplicates, as read_mtx does."""
    key = np.unique(r.astype(np.int64) * cols + c.astype(np.int64))
    return COOMatrix(rows, cols, (key // cols).astype(np.int32), (key % cols).astype(np.int32))


def uniform_matrix(rows: int, cols: int, draws: int, seed: int) -> COOMatrix:
    """`draws` i.i.d. uniform positions, duplicates dropped."""
    g = np.random.default_rng(seed)
    return normalise(rows, cols, g.integers(0, rows, draws), g.integers(0, cols, draws))


def _powerlaw_weights(g, n: int, gamma: float) -> np.ndarray:
    u = g.random(n)
    return (1.0 - u) ** (-1.0 / (gamma - 1.0))


def _symmetric_from_degrees(g, n: int, half_deg: np.ndarray, band: int | None) -> COOMatrix:
    src = np.repeat(np.arange(n, dtype=np.int64), half_deg)
    if band is None:
        dst = g.integers(0, n, src.size)
    else:
        off = g.integers(1, band + 1, src.size) * np.where(g.random(src.size) < 0.5, -1, 1)
        dst = src + off
        dst = np.where((dst < 0) | (dst >= n), src - off, dst)
    keep = (dst != src) & (dst >= 0) & (dst < n)
    src, dst = src[keep], dst[keep]
    return normalise(n, n, np.concatenate([src, dst]), np.concatenate([dst, src]))


def _calibrated(g_seed: int, n: int, gamma: float, max_deg: int, target_nnz: int,
                band: int | None) -> COOMatrix:
    scale = target_nnz / (2.0 * n)
    coo = None
    for _ in range(6):
        g = np.random.default_rng(g_seed)
        w = _powerlaw_weights(g, n, gamma)
        w = w / w.mean()
        # a node's degree is its own draws plus about `scale` incoming ones
        cap = max(1, max_deg - int(round(scale)))
        half = np.minimum(np.rint(w * scale).astype(np.int64), cap)
        half = np.maximum(half, 0)
        coo = _symmetric_from_degrees(g, n, half, band)
        if abs(coo.nnz - target_nnz) <= 0.005 * target_nnz:
            break
        scale *= target_nnz / max(coo.nnz, 1)
    return coo


def banded_powerlaw(n: int = 8219, target_nnz: int = 242_000, gamma: float = 2.3, max_deg: int = 400,
                    band: int = 150, seed: int = 2) -> COOMatrix:
    """Symmetric, empty diagonal, power-law degrees, neighbours within +-band."""
    return _calibrated(seed, n, gamma, max_deg, target_nnz, band)


def uniform_powerlaw(n: int = 16706, target_nnz: int = 396_000, gamma: float = 2.2, max_deg: int = 360,
                     seed: int = 3) -> COOMatrix:
    """Symmetric, empty diagonal, power-law degrees, uniform neighbour ids."""
    return _calibrated(seed, n, gamma, max_deg, target_nnz, None)


def _is_prime(x: int) -> bool:
    if x < 2:
        return False
    for p in range(2, int(math.isqrt(x)) + 1):
        if x % p == 0:
            return False
    return True


def _near_prime(x: int) -> int:
    while not _is_prime(x):
        x += 1
    return x


def _near_smooth5(x: int) -> int:
    while True:
        y = x
        for p in (2, 3, 5):
            while y % p == 0:
                y //= p
        if y == 1:
            return x
        x += 1


def batch_dims(count: int = 64, lo: int = 500, hi: int = 12000, seed: int = 4):
    """(rows, cols, density) triples: dims log-uniform in [lo, hi], half moved
    to the next prime and half to the next 2^a 3^b 5^c; densities log-uniform
    in [1e-4, 1e-2]."""
    g = np.random.default_rng(seed)
    out = []
    for i in range(count):
        dims = []
        for _ in range(2):
            x = int(round(math.exp(g.uniform(math.log(lo), math.log(hi)))))
            dims.append(_near_prime(x) if i % 2 == 0 else _near_smooth5(x))
        dens = math.exp(g.uniform(math.log(1e-4), math.log(1e-2)))
        out.append((dims[0], dims[1], dens))
    return out


def batch_matrices(count: int = 64, seed: int = 4) -> list[COOMatrix]:
    mats = []
    for i, (r, c, d) in enumerate(batch_dims(count, seed=seed)):
        draws = max(1, int(round(r * c * d)))
        mats.append(uniform_matrix(r, c, draws, seed * 100003 + i))
    return mats


def config_matrix(name: str) -> COOMatrix:
    """The benchmark workloads by name."""
    if name == "uniform_3001x2048":
        return uniform_matrix(3001, 2048, 30_730, seed=1)
    if name == "banded_powerlaw_8219":
        return banded_powerlaw()
    if name == "uniform_powerlaw_16706":
        return uniform_powerlaw()
    if name == "uniform_powerlaw_40421":
        return uniform_powerlaw(n=40421, target_nnz=351_000, gamma=2.2, max_deg=360, seed=5)
    raise KeyError(name)


CONFIGS = ("uniform_3001x2048", "banded_powerlaw_8219", "uniform_powerlaw_16706", "uniform_powerlaw_40421")
