"""Exact PCA -- TEST INFRASTRUCTURE ONLY (the checker of the GPU PCA).

The FP64 ground truth of scanpy's `pp.pca` semantics as
crates/scrust-core/src/pca.rs:74-216 reports them: components are the
leading right singular vectors of the (optionally centred) cells x genes
matrix from numpy's LAPACK SVD in float64; the largest-magnitude loading of
each component is made positive (pca.rs:497-519); the explained variance is
S^2 / (n - 1) when centred and each score column's population variance when
not (pca.rs:171-200); ratios are over the sum of every gene's variance, ddof
1 centred and 0 not (pca.rs:227-255).  Only the tests call it.
"""

from __future__ import annotations

import numpy as np


def exact_pca(dense, n_components: int, zero_center: bool = True):
    """(embedding (n, k) f64, components (k, g) f64, variance (k,), ratio (k,))."""
    x = np.asarray(dense, dtype=np.float64)
    n = x.shape[0]
    mean = x.mean(axis=0)
    xc = x - mean if zero_center else x
    u, s, vt = np.linalg.svd(xc, full_matrices=False)
    comps = vt[:n_components]
    emb = u[:, :n_components] * s[:n_components]
    for c in range(n_components):
        j = int(np.argmax(np.abs(comps[c])))  # first largest magnitude
        if comps[c, j] < 0:
            comps[c] = -comps[c]
            emb[:, c] = -emb[:, c]
    ddof = 1.0 if zero_center else 0.0
    sums = x.sum(axis=0)
    squares = (x * x).sum(axis=0)
    total = float(np.sum(np.maximum(squares - sums * sums / n, 0.0) / (n - ddof)))
    if zero_center:
        var = s[:n_components] ** 2 / (n - 1)
    else:
        var = emb.var(axis=0)
    return emb, comps, var, var / total if total > 0 else np.zeros_like(var)


def correlation(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    a = a - a.mean()
    b = b - b.mean()
    return float((a * b).sum() / np.sqrt((a * a).sum() * (b * b).sum()))
