"""Leiden, Louvain and modularity on the GPU (scrust_cuda_leiden / _louvain /
_modularity) against the reference's own cluster tests
(crates/scrust-core/src/cluster.rs, tests module) and against the oracle's
sequential restatement of cluster.rs.

The GPU moves nodes in parallel rounds, so its partitions are its own
(deterministic for a seed), not the sequential queue's.  They are held to the
reference's exact bars on its small graphs (clique recovery, hand-computed
modularity, label order, connectedness, resolution monotonicity, errors) and,
on kNN graphs of clustered cells, to the restatement's modularity within
Q_TOL and to the planted clusters by adjusted Rand index.
"""

from __future__ import annotations

import numpy as np
import pytest

import cluster_cases as cc

pytestmark = pytest.mark.gpu

Q_TOL = 0.01       # modularity(GPU) >= modularity(sequential restatement) - Q_TOL on kNN graphs
EXACT_TOL = 1e-12  # modularity of given labels, GPU against the f64 restatement


@pytest.fixture(scope="module")
def scrust(built_library):
    from mrustsc_gb300 import _scrust

    assert _scrust.gpu_available(), "these tests need an sm_103a GPU"
    return _scrust


def leiden(scrust, g, resolution=1.0, n_iterations=2, seed=0):
    return scrust.leiden(*g, resolution, n_iterations, seed, "auto")


def louvain(scrust, g, resolution=1.0, seed=0):
    return scrust.louvain(*g, resolution, seed, "auto")


def u32(labels):
    return np.asarray(labels, np.uint32)


def knn_graph(scrust, n, clusters, seed, d=20, k=15):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-4.0, 4.0, size=(clusters, d)).astype(np.float32)
    truth = rng.integers(0, clusters, n)
    x = (centres[truth] + rng.standard_normal((n, d)).astype(np.float32)).astype(np.float32)
    _, _, (ip, ix, vl, n_cols) = scrust.neighbors_graph(x, k)
    return (ip, ix, vl, n_cols), truth


def test_modularity_matches_hand_computed_values(scrust, oracle):
    g = cc.barbell()
    cases = [([0, 0, 0, 1, 1, 1], 1.0, 6 / 7 - 0.5), ([0] * 6, 1.0, 0.0),
             ([0, 1, 2, 3, 4, 5], 1.0, -sum((k / 14.0) ** 2 for k in (2, 2, 3, 3, 2, 2))),
             ([0, 0, 0, 1, 1, 1], 2.0, 6 / 7 - 1.0)]
    for labels, res, want in cases:
        got = scrust.modularity(*g, u32(labels), res)
        assert abs(got - want) < EXACT_TOL
        assert abs(got - oracle.modularity(*g, labels, resolution=res)) < EXACT_TOL
    # (A + A^T) / 2: the one-sided barbell at weight 2 is the barbell
    assert abs(scrust.modularity(*cc.half_barbell(), u32([0, 0, 0, 1, 1, 1]), 1.0) - (6 / 7 - 0.5)) < EXACT_TOL


@pytest.mark.parametrize("algorithm", ["leiden", "louvain"])
def test_recovers_disconnected_cliques(scrust, algorithm):
    g = cc.disconnected_cliques(4, 8)
    labels, q, nc = leiden(scrust, g) if algorithm == "leiden" else louvain(scrust, g)
    assert nc == 4
    for c in range(4):
        assert len(set(labels[c * 8:(c + 1) * 8].tolist())) == 1
    assert len(set(labels.tolist())) == 4
    assert abs(q - 0.75) < 1e-12  # four equal disconnected cliques: 1 - 4 * (1/4)^2


def test_leiden_no_worse_than_louvain_and_reported_modularity(scrust):
    g = cc.disconnected_cliques(6, 5)
    for seed in range(4):
        assert leiden(scrust, g, seed=seed)[1] >= louvain(scrust, g, seed=seed)[1] - 1e-9
    g = cc.disconnected_cliques(5, 6)
    labels, q, _ = leiden(scrust, g, seed=3)
    assert abs(q - scrust.modularity(*g, labels, 1.0)) < EXACT_TOL


def test_deterministic_resolution_and_label_order(scrust):
    g = cc.disconnected_cliques(4, 7)
    a, qa, _ = leiden(scrust, g, seed=11)
    b, qb, _ = leiden(scrust, g, seed=11)
    np.testing.assert_array_equal(a, b)
    assert qa == qb
    g = cc.disconnected_cliques(4, 10)
    previous = 0
    for res in (0.25, 0.5, 1.0, 2.0, 4.0):
        _, _, nc = leiden(scrust, g, resolution=res)
        assert nc >= previous
        previous = nc
    labels, _, nc = leiden(scrust, cc.two_cliques_12_and_3())
    assert nc == 2 and labels[3] == 0 and labels[0] == 1


def test_communities_are_internally_connected(scrust):
    g = cc.disconnected_cliques(3, 9)
    labels, _, nc = leiden(scrust, g, seed=5)
    for c in range(nc):
        assert cc.is_connected(g[0], g[1], g[2], np.nonzero(labels == c)[0])


def test_rejects_degenerate_input(scrust):
    empty = (np.zeros(1, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32), 0)
    for call in (lambda: leiden(scrust, empty), lambda: louvain(scrust, empty)):
        with pytest.raises(ValueError):
            call()
    negative = (np.array([0, 1, 2], np.uint32), np.array([1, 0], np.uint32), np.array([-1, -1], np.float32), 2)
    with pytest.raises(ValueError, match="finite and non-negative"):
        leiden(scrust, negative)
    g = cc.disconnected_cliques(2, 3)
    for kwargs in ({"resolution": 0.0}, {"resolution": float("nan")}, {"n_iterations": 0}):
        with pytest.raises(ValueError):
            leiden(scrust, g, **kwargs)
    with pytest.raises(ValueError):
        louvain(scrust, g, resolution=0.0)
    edgeless = (np.zeros(3, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32), 2)
    with pytest.raises(ValueError, match="positive weight"):
        leiden(scrust, edgeless)
    rectangular = (np.array([0, 1], np.uint32), np.array([2], np.uint32), np.array([1.0], np.float32), 4)
    with pytest.raises(ValueError):
        leiden(scrust, rectangular)
    with pytest.raises(ValueError, match="labels, one per node"):
        scrust.modularity(*g, u32([0, 0]), 1.0)
    with pytest.raises(ValueError, match="below the node count"):
        scrust.modularity(*cc.barbell(), u32([0, 1, 2, 3, 4, 2**32 - 1]), 1.0)
    with pytest.raises(ValueError, match="1-D numpy array of uint32"):
        scrust.modularity(*cc.barbell(), [0, 0, 0, 1, 1, 1], 1.0)


@pytest.mark.parametrize("n,clusters,seed", [(3000, 12, 1), (20000, 40, 2)])
def test_knn_graph_modularity_against_the_sequential_restatement(scrust, oracle, n, clusters, seed):
    g, truth = knn_graph(scrust, n, clusters, seed)
    labels, q, nc = leiden(scrust, g, seed=seed)
    o_labels, o_q, _ = oracle.leiden(*g, seed=seed)
    assert q >= o_q - Q_TOL, (q, o_q)
    assert abs(q - oracle.modularity(*g, labels)) < 1e-9
    assert cc.adjusted_rand_index(labels, truth) > 0.9
    assert cc.adjusted_rand_index(labels, o_labels) > 0.85
    l_labels, l_q, _ = louvain(scrust, g, seed=seed)
    o_lq = oracle.louvain(*g, seed=seed)[1]
    assert l_q >= o_lq - Q_TOL, (l_q, o_lq)
    # labels by descending size
    sizes = np.bincount(labels, minlength=nc)
    assert np.all(np.diff(sizes) <= 0) and sizes.min() > 0


def test_knn_graph_communities_are_connected_and_repeatable(scrust):
    g, _ = knn_graph(scrust, 5000, 16, 3)
    a, qa, nc = leiden(scrust, g, seed=7)
    b, qb, _ = leiden(scrust, g, seed=7)
    np.testing.assert_array_equal(a, b)
    assert qa == qb
    for c in range(nc):
        assert cc.is_connected(g[0], g[1], g[2], np.nonzero(a == c)[0])
