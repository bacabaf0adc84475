"""Parity at the benchmark workloads' full sizes, against the C oracle.

* 1,000,000 x 50, k = 15, 200 clusters, 1% duplicates (the precision form):
  10,000 random rows plus every row with a neighbour at distance 0 plus every
  row whose 15th and 16th neighbours are within 1e-5 relative, against the
  FP64 exact kNN (ids bit-exact, lowest index on ties; distances within 1e-6
  relative, zeros exact); and the whole 1M connectivities CSR against the
  oracle's restatement of crates/scrust-core/src/neighbors.rs:208-372 on the
  same kNN graph (structure bit-exact, values within 1e-5 absolute).
* 64 samples, 674k cells (the batching form, no reference counterpart):
  sampled rows of every sample against the FP64 kNN of that sample.
* A 500,000 x 50 atlas with a few hundred Poisson requests (the serving
  form, no reference counterpart): sampled query rows of every request
  against the FP64 query-versus-atlas kNN, and their connectivity rows
  against the oracle's directed weights.
"""

from __future__ import annotations

import numpy as np
import pytest

from mrustsc_gb300 import synthetic

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def scrust(built_library):
    from mrustsc_gb300 import _scrust

    assert _scrust.gpu_available(), "these tests need an sm_103a GPU"
    return _scrust


@pytest.fixture(scope="module")
def parity(oracle):
    from oracle import parity as p

    return p


def test_precision_workload_at_one_million_cells(scrust, parity):
    x = synthetic.precision_scale(seed=0)
    n, k = x.shape[0], 15
    idx, dist, conn = scrust.neighbors_graph(x, k, form="tensor")
    assert not np.any(idx == np.arange(n, dtype=np.uint32)[:, None])
    assert np.all(np.diff(dist, axis=1) >= 0)
    _, dist16 = scrust.knn(x, k + 1, "auto", form="tensor")
    rows, kinds = parity.select_rows(n, dist, dist16, n_random=10_000, seed=0)
    assert kinds["random"] == 10_000 and kinds["zero_distance"] >= 10_000
    rep = parity.knn_rows_report(x, k, idx, dist, rows)
    assert parity.knn_rows_ok(rep), rep
    crep = parity.connectivities_report(idx, dist, conn)
    assert parity.connectivities_ok(crep), crep


def test_batching_workload_every_sample(scrust, parity):
    from oracle import oracle

    samples = synthetic.batch_samples(seed=0)
    k = 15
    out = scrust.knn_batch(samples, k, "auto")
    rng = np.random.default_rng(1)
    for s, (x, (idx, dist)) in enumerate(zip(samples, out)):
        rows = np.unique(np.concatenate([rng.choice(len(x), min(len(x), 64), replace=False),
                                         np.nonzero(dist[:, 0] == 0)[0][:64]]))
        rep = parity.knn_rows_report(x, k, idx, dist, rows)
        assert parity.knn_rows_ok(rep), (s, rep)
    # one whole sample, every row
    x, (idx, dist) = samples[7], out[7]
    oi, _, od = oracle.knn_fp64(x, k)
    np.testing.assert_array_equal(idx, oi)


def test_serving_workload_against_a_500k_atlas(parity, built_library):
    from mrustsc_gb300 import serving

    atlas, centres = synthetic.serving_atlas(seed=0, m=500_000, d=50)
    times, counts = synthetic.poisson_arrivals(200.0, 1.5, seed=1)
    assert len(counts) >= 200
    k = 15
    rng = np.random.default_rng(2)
    picked_q, picked_i, picked_d = [], [], []
    with serving.Server(atlas, k, slots=2) as sv:
        tickets = []
        queries = [synthetic.serving_queries(centres, int(c), seed=100 + i) for i, c in enumerate(counts)]
        for x in queries:
            tickets.append(sv.submit(x))
        for x, t in zip(queries, tickets):
            idx, dist, (indptr, cols, vals), _ = sv.wait(t)
            rows = np.sort(rng.choice(len(x), min(len(x), 4), replace=False))
            ep, ec, ev = parity.query_rows_expected(idx[rows], dist[rows])
            for j, r in enumerate(rows):
                np.testing.assert_array_equal(cols[indptr[r]:indptr[r + 1]], ec[ep[j]:ep[j + 1]])
                np.testing.assert_allclose(vals[indptr[r]:indptr[r + 1]], ev[ep[j]:ep[j + 1]], atol=1e-5, rtol=0)
            picked_q.append(x[rows])
            picked_i.append(idx[rows])
            picked_d.append(dist[rows])
        st = sv.stats()
    assert st["requests"] == len(counts)
    rep = parity.cross_rows_report(np.concatenate(picked_q), atlas, k, np.concatenate(picked_i),
                                   np.concatenate(picked_d))
    assert rep["exact_rows"] == rep["rows"] and rep["max_rel_dist_err"] <= parity.DIST_RTOL, rep
    assert rep["zero_distances_exact"]
