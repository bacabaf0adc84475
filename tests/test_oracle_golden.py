"""The oracle is pinned against the reference's own known answers before it is
trusted as the checker of the CUDA path.

Sources: crates/scrust-core/src/neighbors.rs:408-590 (line, grid, tiling,
argument rejection, symmetry, scanpy golden vectors) and
crates/scrust-gpu/src/kernels/knn.rs:339-415 (Metal cases), plus the FP64
recipe and the fuzzy-union recipe of tests/test_neighbors_audit.py.
"""

from __future__ import annotations

import json
import pathlib

import numpy as np
import pytest
import scipy.sparse as sp

import refdata

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "scanpy_reference_embedding_300x20.json"


def test_line_neighbours_are_adjacent(oracle):
    idx, dist = oracle.knn_reference_cpu(refdata.line(6), 2)
    assert idx[0].tolist() == [1, 2]
    assert dist[0].tolist() == [1.0, 2.0]
    assert idx[2].tolist() == [1, 3]  # tie at distance 1 -> smaller id
    assert idx[5].tolist() == [4, 3]


def test_grid_neighbours_follow_the_lattice(oracle):
    idx, dist = oracle.knn_reference_cpu(refdata.grid(3), 4)
    assert idx[4].tolist() == [1, 3, 5, 7]
    assert idx[0].tolist() == [1, 3, 4, 2]
    assert abs(dist[0, 2] - np.sqrt(2.0)) < 1e-6
    assert abs(dist[0, 3] - 2.0) < 1e-6


def test_tiling_does_not_change_the_result(oracle):
    x = refdata.reference_embedding(200, 8, 7)
    a = oracle.knn_reference_cpu(x, 10, tile_rows=200)
    b = oracle.knn_reference_cpu(x, 10, tile_rows=7)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("k", [0, 6, 7])
def test_rejects_degenerate_k(oracle, k):
    with pytest.raises(oracle.OracleError):
        oracle.knn_reference_cpu(refdata.line(6), k)


@pytest.mark.parametrize("shape", [(0, 4), (5, 0)])
def test_rejects_empty_embeddings(oracle, shape):
    with pytest.raises(oracle.OracleError):
        oracle.knn_reference_cpu(np.zeros(shape, np.float32), 3)


def test_connectivities_reject_a_degenerate_graph(oracle):
    with pytest.raises(oracle.OracleError):
        oracle.connectivities(np.zeros((0, 3), np.uint32), np.zeros((0, 3), np.float32))
    with pytest.raises(oracle.OracleError):
        oracle.connectivities(np.array([[1], [9]], np.uint32), np.ones((2, 1), np.float32))


def test_connectivities_are_symmetric_with_an_empty_diagonal(oracle):
    idx, dist = oracle.knn_reference_cpu(refdata.reference_embedding(120, 5, 3), 10)
    indptr, cols, vals, n = oracle.connectivities(idx, dist)
    m = sp.csr_matrix((vals, cols, indptr), shape=(n, n)).toarray()
    assert np.all(np.diag(m) == 0)
    np.testing.assert_allclose(m, m.T, atol=1e-6)
    assert vals.min() > 0 and vals.max() <= 1
    for r in range(n):
        row = cols[indptr[r]:indptr[r + 1]]
        assert np.all(np.diff(row.astype(np.int64)) > 0)


def test_matches_scanpy_golden_vectors(oracle):
    g = json.loads(GOLDEN.read_text())
    e = g["embedding"]
    x = refdata.reference_embedding(e["n_cells"], e["n_dims"], e["seed"])
    idx, dist = oracle.knn_reference_cpu(x, g["k"])
    for cell, expected in zip(g["sample_cells"], g["scanpy_neighbors"]):
        shared = len(set(idx[cell].tolist()) & set(expected))
        assert shared * 10 >= g["k"] * 9, f"cell {cell}: {shared}"
    indptr, cols, vals, n = oracle.connectivities(idx, dist)
    for cell, row in zip(g["sample_cells"], g["scanpy_connectivity_rows"]):
        ours = dict(zip(cols[indptr[cell]:indptr[cell + 1]].tolist(), vals[indptr[cell]:indptr[cell + 1]].tolist()))
        for c, v in row:
            if c in ours:
                assert abs(ours[c] - v) <= 1e-3 * abs(v), (cell, c)
    assert len(vals) == g["nnz"]
    assert abs(float(vals.sum(dtype=np.float32)) - g["weight_sum"]) <= 1e-3 * g["weight_sum"]
    assert abs(float((vals * vals).sum(dtype=np.float32)) - g["weight_square_sum"]) <= 1e-3 * g["weight_square_sum"]


@pytest.mark.parametrize(("n", "d", "k"), [(64, 8, 1), (100, 5, 7), (257, 3, 15), (300, 32, 16)])
def test_metal_twin_agrees_with_cpu_path_on_random_embeddings(oracle, n, d, k):
    x = refdata.random_embedding(n, d, n)
    a_idx, a_dist = oracle.knn_metal_twin(x, k)
    b_idx, b_dist = oracle.knn_reference_cpu(x, k)
    np.testing.assert_array_equal(a_idx, b_idx)
    np.testing.assert_allclose(a_dist, b_dist, rtol=1e-5, atol=1e-6)


def test_metal_twin_line_and_duplicates(oracle):
    idx, dist = oracle.knn_metal_twin(refdata.line(50), 2)
    assert idx[10].tolist() == [9, 11] and dist[10].tolist() == [1.0, 1.0]
    assert idx[0].tolist() == [1, 2] and dist[0].tolist() == [1.0, 2.0]
    x = np.zeros((41, 2), np.float32)
    x[40, 0] = 100.0
    idx, _ = oracle.knn_metal_twin(x, 3)
    assert idx[5].tolist() == [0, 1, 2]
    assert idx[0].tolist() == [1, 2, 3]


def test_fp64_oracle_matches_the_audit_recipe(oracle):
    x = refdata.audit_embedding(120, 6, 5)
    x[20:30] = x[20]
    ei, ed = oracle.exact_knn_numpy(x, 14)
    fi, fd, _ = oracle.knn_fp64(x, 14)
    np.testing.assert_array_equal(ei, fi)
    np.testing.assert_allclose(ed, fd, rtol=0, atol=1e-12)


def test_fuzzy_union_recipe_is_bit_exact(oracle):
    """tests/test_neighbors_audit.py:297-334 with the oracle's own sigmas and rhos."""
    x = refdata.audit_embedding()
    idx, dist = oracle.knn_fp64(x, 14)[0], oracle.knn_fp64(x, 14)[2]
    sig, rho = oracle.smooth_knn(dist)
    n, k = idx.shape
    offsets = dist - rho[:, None]
    with np.errstate(over="ignore"):
        strengths = np.where(offsets <= 0.0, np.float32(1.0),
                             np.exp(-(offsets / sig[:, None]))).astype(np.float32)
    weights = oracle.directed_weights(idx, dist)
    np.testing.assert_allclose(weights, strengths, rtol=2e-7, atol=0)
    directed = sp.csr_matrix((weights.ravel(), idx.ravel().astype(np.int64), np.arange(0, n * k + 1, k)),
                             shape=(n, n))
    directed.eliminate_zeros()
    union = sp.csr_matrix(directed + directed.T - directed.multiply(directed.T))
    union.sort_indices()
    indptr, cols, vals, _ = oracle.connectivities(idx, dist)
    np.testing.assert_array_equal(union.indptr, indptr)
    np.testing.assert_array_equal(union.indices, cols)
    np.testing.assert_array_equal(union.data.astype(np.float32), vals)


def test_unrolled_sum_order(oracle):
    xs = np.array([1e8, 1.0, -1e8, 1.0, 3.0, 5.0, 7.0, 11.0, 13.0, 17.0, 19.0], np.float32)
    p = [np.float32(0)] * 8
    for i in range(8):
        p[i] = np.float32(p[i] + xs[i])
    acc = np.float32(0)
    for a, b in ((0, 4), (1, 5), (2, 6), (3, 7)):
        acc = np.float32(acc + np.float32(p[a] + p[b]))
    for v in xs[8:]:
        acc = np.float32(acc + v)
    assert oracle.unrolled_sum(xs) == acc


def test_smooth_knn_floors(oracle):
    """Row-mean floor when rho > 0, global-mean floor when rho == 0
    (tests/test_neighbors_audit.py:251-291)."""
    x = refdata.audit_embedding(200, 6, 4) * 10
    x[:20] = x[0]
    _, _, dist = oracle.knn_fp64(x, 14)
    sig, rho = oracle.smooth_knn(dist)
    assert np.count_nonzero(rho == 0) == 20
    mean = oracle.unrolled_sum(dist) / np.float32(dist.size)
    np.testing.assert_array_equal(sig[rho == 0], np.maximum(sig[rho == 0], np.float32(1e-3) * mean))
