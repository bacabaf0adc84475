"""The UMAP oracle (a C restatement of crates/scrust-core/src/umap.rs) against
the reference's own UMAP tests: umap-learn's fitted-curve table, cluster
separation, the zero-negative-rate collapse, seed reproducibility, the
scanpy neighbourhood check on the 80-cell golden graph, and the argument
errors.  CPU only."""

from __future__ import annotations

import numpy as np
import pytest

import umap_cases as uc


def test_fitted_curve_matches_umap_learn(oracle):
    g = uc.golden()
    tol = g["bars"]["fit_ab_relative_tolerance"]
    for min_dist, spread, a_ref, b_ref in g["fit_ab_table"]:
        a, b = oracle.fit_ab_params(min_dist, spread)
        assert abs(a - a_ref) <= tol * abs(a_ref) and abs(b - b_ref) <= tol * abs(b_ref), (min_dist, spread, a, b)


def test_zero_negative_rate_collapses_each_cluster(oracle):
    y = oracle.umap(*uc.two_clusters(6), n_epochs=30, negative_sample_rate=0)
    within, _ = uc.separation(y, 6)
    assert within < 1e-2


@pytest.mark.parametrize("n_components", [1, 2, 3])
def test_shape_and_finite(oracle, n_components):
    y = oracle.umap(*uc.two_clusters(20), n_components=n_components, n_epochs=500)
    assert y.shape == (40, n_components) and np.isfinite(y).all()


def test_clusters_separate_and_seeds_reproduce(oracle):
    g = uc.two_clusters(25)
    y = oracle.umap(*g, n_epochs=500, seed=0)
    within, between = uc.separation(y, 25)
    assert between > 5 * within
    a = oracle.umap(*uc.two_clusters(20), n_epochs=500, seed=42)
    b = oracle.umap(*uc.two_clusters(20), n_epochs=500, seed=42)
    np.testing.assert_array_equal(a, b)
    c = oracle.umap(*g, n_epochs=500, seed=1)
    d = oracle.umap(*g, n_epochs=500, seed=2)
    assert not np.array_equal(c, d)
    within, between = uc.separation(d, 25)
    assert between > 5 * within


def test_neighbourhoods_agree_with_scanpy(oracle):
    g = uc.golden()
    graph = uc.symmetric_from_edges(g["n_cells"], g["edges_upper"])
    y = oracle.umap(*graph, n_epochs=g["bars"]["epochs"], seed=g["bars"]["seed"])
    assert uc.scanpy_preserved_fraction(y) >= g["bars"]["preserved_min_fraction"]


def test_rejects_degenerate_input(oracle):
    g = uc.two_clusters(4)
    with pytest.raises(oracle.OracleError):
        oracle.umap(*g, n_epochs=0)
    with pytest.raises(oracle.OracleError):
        oracle.umap(*g, n_components=0)
    with pytest.raises(oracle.OracleError):
        oracle.umap(np.zeros(1, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32), 0)
    with pytest.raises(oracle.OracleError):
        oracle.umap(*uc.csr_parts(np.zeros((3, 3), np.float32)))
