"""Seeded synthetic embeddings with the shapes and value distributions of the
benchmark workloads (no public dataset is used).

A Gaussian mixture stands in for a PCA embedding: cluster centres uniform in
[-5, 5]^D, per-dimension standard deviation 2 / sqrt(i) for i = 1..D (a
decaying PCA spectrum), exact duplicates that copy a random earlier row, and
near-duplicates that add N(0, 1e-4) to such a copy.
"""

from __future__ import annotations

import numpy as np


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def mixture(n: int, d: int = 50, clusters: int = 8, dup_frac: float = 0.01, near_dup_frac: float = 0.0,
            seed: int = 0, centres: np.ndarray | None = None) -> np.ndarray:
    """(n, d) float32 rows drawn from the mixture, with duplicate rows mixed in."""
    rng = _rng(seed)
    if centres is None:
        centres = rng.uniform(-5.0, 5.0, size=(clusters, d)).astype(np.float32)
    std = (2.0 / np.sqrt(np.arange(1, d + 1, dtype=np.float64))).astype(np.float32)
    labels = rng.integers(0, len(centres), n)
    x = rng.standard_normal((n, d), dtype=np.float32)
    x *= std
    x += centres[labels]
    n_dup = int(round(dup_frac * n))
    n_near = int(round(near_dup_frac * n))
    if n > 1 and (n_dup or n_near):
        rows = rng.choice(np.arange(1, n), size=min(n - 1, n_dup + n_near), replace=False)
        dup_rows = np.sort(rows[:n_dup])
        near_rows = np.sort(rows[n_dup:])
        for r in dup_rows:
            x[r] = x[int(rng.integers(0, r))]
        noise = rng.normal(0.0, 1e-4, size=(len(near_rows), d)).astype(np.float32)
        for t, r in enumerate(near_rows):
            x[r] = x[int(rng.integers(0, r))] + noise[t]
    return x


def plain_small(seed: int = 0) -> np.ndarray:
    """2,638 x 50, 8 clusters, 1% exact duplicates (k = 15)."""
    return mixture(2638, 50, clusters=8, dup_frac=0.01, seed=seed)


def plain_scale(seed: int = 0, n: int = 100_000) -> np.ndarray:
    """100,000 x 50, 40 clusters, 0.5% duplicates and 0.5% near-duplicates (k = 30)."""
    return mixture(n, 50, clusters=40, dup_frac=0.005, near_dup_frac=0.005, seed=seed)


def precision_scale(seed: int = 0, n: int = 1_000_000) -> np.ndarray:
    """1,000,000 x 50, 200 clusters, 1% duplicates (k = 15)."""
    return mixture(n, 50, clusters=200, dup_frac=0.01, seed=seed)


def batch_samples(seed: int = 0, n_samples: int = 64, lo: int = 500, hi: int = 50_000, d: int = 50):
    """List of per-sample embeddings: sizes log-uniform in [lo, hi], 4-20 clusters each."""
    rng = _rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), n_samples)).astype(np.int64)
    clusters = rng.integers(4, 21, n_samples)
    return [mixture(int(sizes[s]), d, clusters=int(clusters[s]), dup_frac=0.01, seed=seed * 1000 + s + 1)
            for s in range(n_samples)]


def serving_atlas(seed: int = 0, m: int = 500_000, d: int = 50, clusters: int = 100):
    """(atlas (m, d) float32, centres) for the query service workload."""
    rng = _rng(seed)
    centres = rng.uniform(-5.0, 5.0, size=(clusters, d)).astype(np.float32)
    return mixture(m, d, dup_frac=0.0, seed=seed + 1, centres=centres), centres


def serving_queries(centres: np.ndarray, q: int, seed: int) -> np.ndarray:
    """q query cells: draws from the atlas clusters plus an N(0, 0.1) shift."""
    x = mixture(q, centres.shape[1], dup_frac=0.0, seed=seed, centres=centres)
    x += _rng(seed + 7).normal(0.0, 0.1, size=x.shape).astype(np.float32)
    return x


def poisson_arrivals(rate: float, duration_s: float, seed: int, lo: int = 1, hi: int = 20_000):
    """(arrival times s, query counts): Poisson arrivals, counts log-uniform in [lo, hi]."""
    rng = _rng(seed)
    times = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration_s:
            break
        times.append(t)
    counts = np.exp(rng.uniform(np.log(lo), np.log(hi + 1), len(times))).astype(np.int64)
    return np.asarray(times), np.clip(counts, lo, hi)
