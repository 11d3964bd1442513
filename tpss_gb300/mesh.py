"""Distorted unit-cube meshes, as the reference builds them (apps/mesh.h:160-200).

`distorted_cube` returns the vertex coordinates (lexicographic, x fastest) of the unit cube with
n cells per direction whose interior vertices are moved as GridTools::distort_random moves
them: in a uniformly random direction, by `factor` times the shortest edge at the vertex;
boundary vertices stay. The random stream is numpy's Philox with the given seed.
"""
from __future__ import annotations

import numpy as np


def distorted_cube(dim: int, n_cells, seed: int, factor: float) -> np.ndarray:
    nc = [int(n) for n in n_cells]
    assert len(nc) == dim and 0.0 <= factor < 0.5, "factor must be in [0, 0.5)"
    nv = [n + 1 for n in nc]
    grids = np.meshgrid(*[np.arange(n) / (n - 1) for n in reversed(nv)], indexing="ij")
    X = np.stack([grids[dim - 1 - d] for d in range(dim)], axis=-1).reshape(-1, dim)
    rng = np.random.Generator(np.random.Philox(seed))
    direction = rng.normal(size=X.shape)
    direction /= np.linalg.norm(direction, axis=1, keepdims=True)
    shortest = 1.0 / max(nc)
    idx = np.indices(list(reversed(nv))).reshape(dim, -1)[::-1].T
    interior = np.all((idx > 0) & (idx < np.array(nc)[None, :]), axis=1)
    X[interior] += factor * shortest * direction[interior]
    return np.ascontiguousarray(X)
