"""Graphs and layout checks of the reference's UMAP tests
(crates/scrust-core/src/umap.rs, tests module), shared by the oracle's CPU
tests and the GPU layout's tests."""

from __future__ import annotations

import json
import pathlib

import numpy as np
import scipy.sparse as sp

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "umap_reference_80_cells.json"


def golden() -> dict:
    return json.loads(GOLDEN.read_text())


def csr_parts(m):
    m = sp.csr_matrix(m)
    m.sort_indices()
    return m.indptr.astype(np.uint32), m.indices.astype(np.uint32), m.data.astype(np.float32), m.shape[1]


def two_clusters(per_cluster: int):
    """Two fully connected blobs joined by one weak bridge (umap.rs two_clusters)."""
    n = 2 * per_cluster
    dense = np.zeros((n, n), np.float32)
    for r in range(n):
        for c in range(n):
            if r != c and (r < per_cluster) == (c < per_cluster):
                dense[r, c] = 1.0
    dense[per_cluster - 1, per_cluster] = 0.01
    dense[per_cluster, per_cluster - 1] = 0.01
    return csr_parts(dense)


def symmetric_from_edges(n: int, edges):
    dense = np.zeros((n, n), np.float32)
    for h, t, w in edges:
        dense[h, t] = w
        dense[t, h] = w
    return csr_parts(dense)


def separation(y, per_cluster: int):
    n = 2 * per_cluster
    d = np.sqrt(((y[:, None, :].astype(np.float64) - y[None, :, :]) ** 2).sum(-1))
    same = (np.arange(n)[:, None] < per_cluster) == (np.arange(n)[None, :] < per_cluster)
    iu = np.triu_indices(n, 1)
    within = d[iu][same[iu]].mean()
    between = d[iu][~same[iu]].mean()
    return within, between


def nearest(y, cell: int, k: int):
    d = np.sqrt(((y.astype(np.float64) - y[cell]) ** 2).sum(-1))
    order = [j for j in np.lexsort((np.arange(len(y)), d)) if j != cell]
    return order[:k]


def scanpy_preserved_fraction(y) -> float:
    g = golden()
    n = g["n_cells"]
    ref = np.asarray(g["scanpy_layout"], np.float32).reshape(n, 2)
    near, wide = g["bars"]["near"], g["bars"]["wide"]
    kept = 0
    for cell in range(n):
        w = set(nearest(y, cell, wide))
        kept += sum(1 for j in nearest(ref, cell, near) if j in w)
    return kept / (n * near)


def trustworthiness(x, y, k: int = 15) -> float:
    """Trustworthiness of a layout (Venna and Kaski, 2001): 1 minus the rank
    penalty of the layout neighbours that are not input neighbours.  numpy,
    small n only."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    n = len(x)
    dx = ((x[:, None, :] - x[None, :, :]) ** 2).sum(-1)
    dy = ((y[:, None, :] - y[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(dx, np.inf)
    np.fill_diagonal(dy, np.inf)
    order_x = np.argsort(dx, axis=1, kind="stable")
    ranks = np.empty_like(order_x)
    ranks[np.arange(n)[:, None], order_x] = np.arange(1, n + 1)[None, :]
    nn_y = np.argsort(dy, axis=1, kind="stable")[:, :k]
    penalty = 0.0
    for i in range(n):
        r = ranks[i, nn_y[i]]
        penalty += np.maximum(r - k, 0).sum()
    return 1.0 - 2.0 / (n * k * (2 * n - 3 * k - 1)) * penalty
