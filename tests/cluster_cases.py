"""Graphs and checks of the reference's community-detection tests
(crates/scrust-core/src/cluster.rs, tests module), shared by the oracle's
CPU tests and the GPU clustering tests."""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def csr_parts(dense):
    m = sp.csr_matrix(np.asarray(dense, np.float32))
    m.sort_indices()
    return m.indptr.astype(np.uint32), m.indices.astype(np.uint32), m.data.astype(np.float32), m.shape[1]


def disconnected_cliques(n_cliques: int, size: int):
    n = n_cliques * size
    d = np.zeros((n, n), np.float32)
    for c in range(n_cliques):
        for a in range(size):
            for b in range(size):
                if a != b:
                    d[c * size + a, c * size + b] = 1.0
    return csr_parts(d)


BARBELL_EDGES = [(0, 1), (0, 2), (1, 2), (3, 4), (3, 5), (4, 5), (2, 3)]


def barbell():
    d = np.zeros((6, 6), np.float32)
    for a, b in BARBELL_EDGES:
        d[a, b] = d[b, a] = 1.0
    return csr_parts(d)


def half_barbell():
    d = np.zeros((6, 6), np.float32)
    for a, b in BARBELL_EDGES:
        d[a, b] = 2.0
    return csr_parts(d)


def two_cliques_12_and_3():
    d = np.zeros((15, 15), np.float32)
    for start, size in ((0, 3), (3, 12)):
        for a in range(start, start + size):
            for b in range(start, start + size):
                if a != b:
                    d[a, b] = 1.0
    return csr_parts(d)


def is_connected(indptr, indices, values, subset) -> bool:
    inside = set(int(v) for v in subset)
    adj = {}
    for r in range(len(indptr) - 1):
        for e in range(indptr[r], indptr[r + 1]):
            if values[e] > 0:
                adj.setdefault(r, []).append(int(indices[e]))
                adj.setdefault(int(indices[e]), []).append(r)
    start = int(subset[0])
    seen, stack = {start}, [start]
    while stack:
        v = stack.pop()
        for u in adj.get(v, []):
            if u in inside and u not in seen:
                seen.add(u)
                stack.append(u)
    return len(seen) == len(inside)


def adjusted_rand_index(a, b) -> float:
    a = np.asarray(a, np.int64)
    b = np.asarray(b, np.int64)
    _, ai = np.unique(a, return_inverse=True)
    _, bi = np.unique(b, return_inverse=True)
    table = np.zeros((ai.max() + 1, bi.max() + 1), np.int64)
    np.add.at(table, (ai, bi), 1)
    comb = lambda x: x * (x - 1) / 2.0  # noqa: E731
    s_ij = comb(table).sum()
    s_a = comb(table.sum(1)).sum()
    s_b = comb(table.sum(0)).sum()
    expected = s_a * s_b / comb(len(a))
    top = 0.5 * (s_a + s_b)
    return 1.0 if top == expected else float((s_ij - expected) / (top - expected))
