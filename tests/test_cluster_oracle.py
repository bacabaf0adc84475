"""The community-detection oracle (a C restatement of
crates/scrust-core/src/cluster.rs) against the reference's own cluster
tests: hand-computed modularity, resolution scaling, clique recovery by
both algorithms, Leiden never below Louvain, reported modularity, seeds,
resolution monotonicity, labels by descending size, symmetrisation, argument
errors and internally connected communities.  CPU only."""

from __future__ import annotations

import numpy as np
import pytest

import cluster_cases as cc


def test_modularity_matches_hand_computed_values(oracle):
    g = cc.barbell()
    assert abs(oracle.modularity(*g, [0, 0, 0, 1, 1, 1]) - (6 / 7 - 0.5)) < 1e-12
    assert abs(oracle.modularity(*g, [0] * 6)) < 1e-12
    alone = -sum((k / 14.0) ** 2 for k in (2, 2, 3, 3, 2, 2))
    assert abs(oracle.modularity(*g, [0, 1, 2, 3, 4, 5]) - alone) < 1e-12
    at_two = oracle.modularity(*g, [0, 0, 0, 1, 1, 1], resolution=2.0)
    assert abs(at_two - (6 / 7 - 1.0)) < 1e-12
    assert abs(oracle.modularity(*cc.half_barbell(), [0, 0, 0, 1, 1, 1]) - (6 / 7 - 0.5)) < 1e-12


@pytest.mark.parametrize("algorithm", ["leiden", "louvain"])
def test_recovers_disconnected_cliques(oracle, algorithm):
    g = cc.disconnected_cliques(4, 8)
    labels, _, nc = oracle.leiden(*g) if algorithm == "leiden" else oracle.louvain(*g)
    assert nc == 4
    for c in range(4):
        assert len(set(labels[c * 8:(c + 1) * 8].tolist())) == 1
    assert len(set(labels.tolist())) == 4


def test_leiden_no_worse_than_louvain_and_reported_modularity(oracle):
    g = cc.disconnected_cliques(6, 5)
    for seed in range(8):
        assert oracle.leiden(*g, seed=seed)[1] >= oracle.louvain(*g, seed=seed)[1] - 1e-9
    g = cc.disconnected_cliques(5, 6)
    labels, q, _ = oracle.leiden(*g, seed=3)
    assert abs(q - oracle.modularity(*g, labels)) < 1e-12


def test_seeds_resolution_and_label_order(oracle):
    g = cc.disconnected_cliques(4, 7)
    a, qa, _ = oracle.leiden(*g, seed=11)
    b, qb, _ = oracle.leiden(*g, seed=11)
    np.testing.assert_array_equal(a, b)
    assert qa == qb
    g = cc.disconnected_cliques(4, 10)
    previous = 0
    for res in (0.25, 0.5, 1.0, 2.0, 4.0):
        _, _, nc = oracle.leiden(*g, resolution=res)
        assert nc >= previous
        previous = nc
    labels, _, nc = oracle.leiden(*cc.two_cliques_12_and_3())
    assert nc == 2 and labels[3] == 0 and labels[0] == 1


def test_communities_are_internally_connected(oracle):
    g = cc.disconnected_cliques(3, 9)
    labels, _, nc = oracle.leiden(*g, seed=5)
    for c in range(nc):
        assert cc.is_connected(g[0], g[1], g[2], np.nonzero(labels == c)[0])


def test_rejects_degenerate_input(oracle):
    empty = (np.zeros(1, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32), 0)
    for call in (lambda: oracle.leiden(*empty), lambda: oracle.louvain(*empty)):
        with pytest.raises(oracle.OracleError):
            call()
    negative = (np.array([0, 1, 2], np.uint32), np.array([1, 0], np.uint32), np.array([-1, -1], np.float32), 2)
    with pytest.raises(oracle.OracleError):
        oracle.leiden(*negative)
    g = cc.disconnected_cliques(2, 3)
    for kwargs in ({"resolution": 0.0}, {"resolution": float("nan")}, {"n_iterations": 0}):
        with pytest.raises(oracle.OracleError):
            oracle.leiden(*g, **kwargs)
    with pytest.raises(oracle.OracleError):
        oracle.louvain(*g, resolution=0.0)
    edgeless = (np.zeros(3, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32), 2)
    with pytest.raises(oracle.OracleError):
        oracle.leiden(*edgeless)
    rectangular = (np.array([0, 1], np.uint32), np.array([2], np.uint32), np.array([1.0], np.float32), 4)
    with pytest.raises(oracle.OracleError):
        oracle.leiden(*rectangular)
    with pytest.raises(oracle.OracleError):
        oracle.modularity(*g, [0, 0])
    with pytest.raises(oracle.OracleError):
        oracle.modularity(*cc.barbell(), [0, 1, 2, 3, 4, 2**32 - 1])
