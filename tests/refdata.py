"""Input generators the reference's own tests use, restated for these tests.

- `reference_embedding`: splitmix64 stream, crates/scrust-core/src/neighbors.rs:380-392
- `line`, `grid`: neighbors.rs:394-406
- `random_embedding`: the LCG of crates/scrust-gpu/src/kernels/knn.rs:317-325
- `audit_embedding`: numpy default_rng normal cloud, tests/test_neighbors_audit.py:47-49
- `pca_scanpy_fixture`, `pca_planted`: the LCG matrices of crates/scrust-core/src/pca.rs's tests
"""

from __future__ import annotations

import numpy as np

_MASK = (1 << 64) - 1


def reference_embedding(n_cells: int, n_dims: int, seed: int) -> np.ndarray:
    state = seed & _MASK
    out = np.empty(n_cells * n_dims, dtype=np.float32)
    for i in range(n_cells * n_dims):
        state = (state + 0x9E3779B97F4A7C15) & _MASK
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
        z ^= z >> 31
        out[i] = np.float32(z >> 40) / np.float32(1 << 24)
    return out.reshape(n_cells, n_dims)


def line(n_cells: int) -> np.ndarray:
    return np.arange(n_cells, dtype=np.float32)[:, None]


def grid(side: int) -> np.ndarray:
    cells = np.arange(side * side)
    return np.stack([cells // side, cells % side], axis=1).astype(np.float32)


def random_embedding(n_cells: int, n_dims: int, seed: int) -> np.ndarray:
    state = (seed * 2 + 1) & _MASK
    out = np.empty(n_cells * n_dims, dtype=np.float32)
    for i in range(n_cells * n_dims):
        state = (state * 6364136223846793005 + 1442695040888963407) & _MASK
        out[i] = np.float32(state >> 40) / np.float32(1 << 24)
    return out.reshape(n_cells, n_dims)


def audit_embedding(n_cells: int = 240, n_dims: int = 10, seed: int = 11) -> np.ndarray:
    return np.random.default_rng(seed).normal(size=(n_cells, n_dims)).astype(np.float32)


class _PcaLcg:
    """The LCG of crates/scrust-core/src/pca.rs's tests: state * 6364136223846793005
    + 1442695040888963407, value (state >> 40) / 2^24 in f64."""

    def __init__(self, seed: int):
        self.state = seed & _MASK

    def next(self) -> float:
        self.state = (self.state * 6364136223846793005 + 1442695040888963407) & _MASK
        return (self.state >> 40) / float(1 << 24)


def pca_scanpy_fixture() -> np.ndarray:
    """300 x 200 counts, four cell groups each raised by 5 in its own block of
    50 genes (pca.rs scanpy_fixture); dense f32."""
    rng = _PcaLcg(42)
    out = np.zeros((300, 200), np.float32)
    for cell in range(300):
        group = cell % 4
        for gene in range(200):
            u = rng.next()
            value = 0.0 if u < 0.6 else float(np.floor(u * 10.0))
            if gene // 50 == group:
                value += 5.0
            out[cell, gene] = value
    return out


def pca_planted() -> np.ndarray:
    """300 x 200: three factors of amplitude 6, 4, 2 on disjoint blocks of 20
    genes with orthogonal cell scores, plus uniform noise (pca.rs planted)."""
    rng = _PcaLcg(7)
    amplitudes = [6.0, 4.0, 2.0]
    scores = [[1.0, 1.0, -1.0, -1.0], [1.0, -1.0, -1.0, 1.0], [1.0, -1.0, 1.0, -1.0]]
    out = np.zeros((300, 200), np.float32)
    for cell in range(300):
        for gene in range(200):
            value = np.float32(rng.next() * 2.0 - 1.0)
            factor = gene // 20
            if factor < 3:
                value = np.float32(value + np.float32(amplitudes[factor] * scores[factor][cell % 4]))
            out[cell, gene] = value
    return out
