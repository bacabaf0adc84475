"""The UMAP layout on the GPU (scrust_cuda_umap) against the reference's own
UMAP tests (crates/scrust-core/src/umap.rs, tests module) and against the
oracle's sequential restatement of umap.rs.

The GPU layout is deterministic (every epoch's moves are computed from the
layout at the epoch's start and summed per cell in a fixed order), so it is
not the sequential sweep's bits.  It is held to the reference's quality bars
(cluster separation, the zero-negative-rate collapse, 80% of scanpy's
neighbourhoods on the 80-cell golden graph), to bit-identical repeat runs,
and to the sequential restatement's trustworthiness within TRUST_TOL.
"""

from __future__ import annotations

import numpy as np
import pytest

import umap_cases as uc
from mrustsc_gb300 import synthetic

pytestmark = pytest.mark.gpu

TRUST_TOL = 0.01  # |trustworthiness(GPU) - trustworthiness(sequential restatement)|, k = 15


@pytest.fixture(scope="module")
def scrust(built_library):
    from mrustsc_gb300 import _scrust

    assert _scrust.gpu_available(), "these tests need an sm_103a GPU"
    return _scrust


def layout(scrust, graph, n_components=2, n_epochs=500, seed=0, negative_sample_rate=5, min_dist=0.5):
    ip, ix, vl, n_cols = graph
    return scrust.umap(ip, ix, vl, n_cols, n_components, n_epochs, min_dist, 1.0, 1.0, negative_sample_rate, seed,
                       "auto")


def test_zero_negative_rate_collapses_each_cluster(scrust):
    """With repulsion off each fully connected cluster collapses.  The
    reference's sequential sweep gets below 1e-2 in 30 epochs; a synchronous
    update sums every pull computed from the same snapshot, which contracts
    such a cluster more slowly, and gets there at the default 200 epochs."""
    y = layout(scrust, uc.two_clusters(6), n_epochs=200, negative_sample_rate=0)
    within, _ = uc.separation(y, 6)
    assert within < 1e-2


@pytest.mark.parametrize("n_components", [1, 2, 3, 16])
def test_shape_and_finite(scrust, n_components):
    y = layout(scrust, uc.two_clusters(20), n_components=n_components)
    assert y.shape == (40, n_components) and np.isfinite(y).all()


def test_clusters_separate_and_seeds_reproduce_bit_for_bit(scrust):
    g = uc.two_clusters(25)
    y = layout(scrust, g, seed=0)
    within, between = uc.separation(y, 25)
    assert between > 5 * within
    a = layout(scrust, uc.two_clusters(20), seed=42)
    b = layout(scrust, uc.two_clusters(20), seed=42)
    np.testing.assert_array_equal(a, b)
    c, d = layout(scrust, g, seed=1), layout(scrust, g, seed=2)
    assert not np.array_equal(c, d)
    within, between = uc.separation(d, 25)
    assert between > 5 * within


def test_neighbourhoods_agree_with_scanpy(scrust):
    g = uc.golden()
    graph = uc.symmetric_from_edges(g["n_cells"], g["edges_upper"])
    y = layout(scrust, graph, n_epochs=g["bars"]["epochs"], seed=g["bars"]["seed"])
    assert uc.scanpy_preserved_fraction(y) >= g["bars"]["preserved_min_fraction"]


def test_trustworthiness_matches_the_sequential_restatement(scrust, oracle):
    x = synthetic.plain_small(seed=0)
    idx, dist, (ip, ix, vl, n) = scrust.neighbors_graph(x, 14)
    y_gpu = scrust.umap(ip, ix, vl, n, 2, 200, 0.5, 1.0, 1.0, 5, 0, "auto")
    y_again = scrust.umap(ip, ix, vl, n, 2, 200, 0.5, 1.0, 1.0, 5, 0, "auto")
    np.testing.assert_array_equal(y_gpu, y_again)
    y_seq = oracle.umap(ip, ix, vl, n, n_epochs=200)
    t_gpu, t_seq = uc.trustworthiness(x, y_gpu, 15), uc.trustworthiness(x, y_seq, 15)
    assert abs(t_gpu - t_seq) <= TRUST_TOL, (t_gpu, t_seq)


def test_tl_umap_surface(built_library):
    from mrustsc_gb300 import pp, tl
    from mrustsc_gb300.anndata_lite import AnnData

    x = synthetic.mixture(600, 20, clusters=4, dup_frac=0.01, seed=3)
    adata = AnnData(np.zeros((600, 2), np.float32), obsm={"X_pca": x})
    pp.neighbors(adata, n_neighbors=15)
    tl.umap(adata, n_epochs=50)
    assert adata.obsm["X_umap"].shape == (600, 2) and adata.obsm["X_umap"].dtype == np.float32


def test_rejects_degenerate_input(scrust):
    g = uc.two_clusters(4)
    with pytest.raises(ValueError):
        layout(scrust, g, n_epochs=0)
    with pytest.raises(ValueError):
        layout(scrust, g, n_components=0)
    with pytest.raises(ValueError):
        layout(scrust, (np.zeros(1, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32), 0))
    with pytest.raises(ValueError):
        layout(scrust, uc.csr_parts(np.zeros((3, 3), np.float32)))
    with pytest.raises(ValueError):
        layout(scrust, g, min_dist=5.0)
