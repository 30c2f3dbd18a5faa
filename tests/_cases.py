"""Seeded case generators shared by the parity tests.

The grid follows the reference's differential tests: n in {3,4,5,7,8,17,100,
500,1000}, three metrics and the LS caps {0,1,7,127,inf}
(tests/cpp/test_cuda_faco.cpp:31-66,136-142), here with EUC_2D integers:
  metric 0 -- candidate rows given in reversed order (the engine must build
              its own distance-ordered LS view),
  metric 1 -- plain uniform integer coordinates,
  metric 2 -- every third point coincides with point 0 (zero distances).
"""
from __future__ import annotations

import numpy as np

N_GRID = (3, 4, 5, 7, 8, 17, 100, 500, 1000)
CAPS = (0, 1, 7, 127, 2**64 - 1)
MNE_LEVELS = (2, 4, 8, 16)


def coordinates(n: int, metric: int, seed: int, box: int = 10**6) -> np.ndarray:
    rng = np.random.default_rng(seed)
    xy = rng.integers(0, box + 1, size=(n, 2), dtype=np.int64).astype(np.int32)
    if metric == 2:
        xy[3::3] = xy[0]
    return xy


def ls_rows(matrix: np.ndarray, width: int, reverse: bool) -> np.ndarray:
    """Nearest `width` nodes by (distance, id); optionally reversed in the row."""
    n = matrix.shape[0]
    rows = np.zeros((n, width), np.uint32)
    for a in range(n):
        order = np.lexsort((np.arange(n), matrix[a]))
        order = order[order != a][:width]
        rows[a] = order[::-1] if reverse else order
    return rows


def ant_tasks(n: int, ants: int, seed: int):
    rng = np.random.default_rng(seed)
    tours = np.stack([rng.permutation(n) for _ in range(ants)]).astype(np.uint32)
    visits = np.stack([rng.permutation(n) for _ in range(ants)]).astype(np.uint32)
    targets = np.array([MNE_LEVELS[a % 4] for a in range(ants)], np.uint32)
    return tours, visits, targets


def uniform_instance(n: int, seed: int, box: int = 10**6) -> np.ndarray:
    """Int coordinates uniform in [0, box]^2 (the spec generator)."""
    rng = np.random.default_rng(seed)
    return rng.integers(0, box + 1, size=(n, 2), dtype=np.int64).astype(np.int32)
