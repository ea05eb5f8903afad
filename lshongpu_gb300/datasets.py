"""Seeded synthetic workloads with the shapes and value distributions of the benchmark
configurations (they stand in for the SIFT / GloVe / GIST files the reference used,
which are not available; no item of those datasets is reproduced).

  clustered(n, d, seed)   mixture of `centers` Gaussian clusters: centres uniform on the
                          unit sphere (from `center_seed`), per-coordinate sigma 0.05,
                          rows L2-normalised; queries use the same centres and seed+1
  sparse_gamma(n, d, seed) nonnegative rows, Bernoulli(0.3) support, Gamma(2, 1) weights
                          (at least one nonzero per row)
"""
from __future__ import annotations

import numpy as np


def centers(d: int, count: int = 1000, center_seed: int = 1234) -> np.ndarray:
    g = np.random.default_rng(center_seed)
    c = g.standard_normal((count, d))
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    return c


def clustered(n: int, d: int, seed: int, count: int = 1000, sigma: float = 0.05, center_seed: int = 1234,
              pad_to: int | None = None, chunk: int = 1 << 18) -> np.ndarray:
    """n unit vectors from the cluster mixture, float32, optionally zero-padded to pad_to."""
    c = centers(d, count, center_seed)
    g = np.random.default_rng(seed)
    width = pad_to or d
    out = np.zeros((n, width), dtype=np.float32)
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        lab = g.integers(0, count, size=m)
        v = c[lab] + sigma * g.standard_normal((m, d))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        out[s:s + m, :d] = v
    return out


def sparse_gamma(n: int, d: int, seed: int, density: float = 0.3, shape: float = 2.0) -> np.ndarray:
    g = np.random.default_rng(seed)
    mask = g.random((n, d)) < density
    empty = ~mask.any(axis=1)
    mask[empty, g.integers(0, d, size=int(empty.sum()))] = True
    vals = g.gamma(shape, 1.0, size=(n, d))
    return np.where(mask, vals, 0.0).astype(np.float32)
