"""Seeded synthetic TSP instances with integer coordinates (TSPLIB EUC_2D),
standing in for the reference's uniform TSP500/TSP1000 dataset rows and for
the clustered workloads of the batch configurations."""
from __future__ import annotations

import numpy as np


def uniform(n: int, seed: int, box: int = 10**6) -> np.ndarray:
    """n points uniform in [0, box]^2 (integers), int32 [n, 2]."""
    rng = np.random.default_rng(seed)
    return rng.integers(0, box + 1, size=(n, 2)).astype(np.int32)


def clustered(n: int, seed: int, *, clusters: tuple[int, int] = (4, 16), sigma: tuple[float, float] = (0.02, 0.08),
              noise: float = 0.2, box: int = 10**6) -> np.ndarray:
    """A mixture of Gaussian clusters (count uniform in `clusters`, each with
    sigma uniform in `sigma` x box) plus a `noise` fraction of uniform points,
    clipped to [0, box]^2 and rounded to integers."""
    rng = np.random.default_rng(seed)
    m = int(rng.integers(clusters[0], clusters[1] + 1))
    centres = rng.uniform(0, box, size=(m, 2))
    sig = rng.uniform(sigma[0], sigma[1], size=m) * box
    n_noise = int(round(noise * n))
    which = rng.integers(0, m, size=n - n_noise)
    pts = centres[which] + rng.normal(size=(n - n_noise, 2)) * sig[which, None]
    pts = np.concatenate([pts, rng.uniform(0, box, size=(n_noise, 2))])
    pts = np.clip(np.rint(pts), 0, box)
    return pts[rng.permutation(n)].astype(np.int32)


def uneven_batch(count: int = 256, n_range: tuple[int, int] = (200, 1000), first_seed: int = 0) -> list:
    """Clustered instances with N uniform in n_range, seed = instance id."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(first_seed + i)
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        out.append(clustered(n, first_seed + i))
    return out


def large_clustered(count: int = 16, first_seed: int = 0) -> list:
    """N uniform in [5000, 10000], 32-64 clusters, coordinates in [0, 10^7]^2."""
    out = []
    for i in range(count):
        rng = np.random.default_rng(10_000 + first_seed + i)
        n = int(rng.integers(5000, 10001))
        out.append(clustered(n, 10_000 + first_seed + i, clusters=(32, 64), box=10**7))
    return out
