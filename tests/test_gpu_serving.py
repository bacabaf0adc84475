"""The query service on the GPU: exact neighbours of each request against a
resident atlas, its directed connectivity rows, and the same result whether
a request is answered alone or batched with others (continuous batching).

No reference counterpart: parity is against an FP64 exact query-versus-
reference restatement and the oracle's smooth_knn / directed weights.
"""

from __future__ import annotations

import threading

import numpy as np
import pytest

from mrustsc_gb300 import synthetic

pytestmark = pytest.mark.gpu

K = 15


@pytest.fixture(scope="module", params=["routed", "swept"])
def world(built_library, request):
    """A service over a 20k-cell atlas, its batches routed to the atlas cells
    (the default) or swept over every atlas tile."""
    import os

    from mrustsc_gb300 import _scrust, serving

    assert _scrust.gpu_available(), "these tests need an sm_103a GPU"
    atlas, centres = synthetic.serving_atlas(seed=3, m=20_000, d=30, clusters=12)
    old = os.environ.get("SCRUST_ROUTED_MIN_QUERIES")
    if request.param == "swept":
        os.environ["SCRUST_ROUTED_MIN_QUERIES"] = str(1 << 40)
    try:
        sv = serving.Server(atlas, K, slots=2, max_batch_cells=4096)
    finally:
        if old is None:
            os.environ.pop("SCRUST_ROUTED_MIN_QUERIES", None)
        else:
            os.environ["SCRUST_ROUTED_MIN_QUERIES"] = old
    yield atlas, centres, sv
    sv.close()


def expected_rows(oracle, idx, dist):
    """Directed weights of query rows (no self to drop: ids are shifted past
    any row index before the oracle sees them), columns ascending."""
    shifted = idx.astype(np.uint64) + (1 << 31)
    w = oracle.directed_weights(shifted.astype(np.uint32), dist)
    indptr = [0]
    cols, vals = [], []
    for i in range(len(idx)):
        keep = w[i] != 0
        order = np.argsort(idx[i][keep], kind="stable")
        cols.extend(idx[i][keep][order].tolist())
        vals.extend(w[i][keep][order].tolist())
        indptr.append(len(cols))
    return np.asarray(indptr, np.uint32), np.asarray(cols, np.uint32), np.asarray(vals, np.float32)


@pytest.mark.parametrize("q", [1, 7, 300, 2500])
def test_requests_are_exact(world, oracle, q):
    atlas, centres, sv = world
    x = synthetic.serving_queries(centres, q, seed=q)
    idx, dist, (indptr, cols, vals), lat = sv.query(x)
    oi, od = oracle.knn_fp64_cross(x, atlas, K)
    np.testing.assert_array_equal(idx, oi)
    rel = np.abs(dist.astype(np.float64) - od) / np.maximum(od, 1e-30)
    assert rel.max() <= 1e-6
    ep, ec, ev = expected_rows(oracle, idx, dist)
    np.testing.assert_array_equal(indptr, ep)
    np.testing.assert_array_equal(cols, ec)
    np.testing.assert_allclose(vals, ev, atol=1e-5, rtol=0)
    assert lat > 0


def test_same_result_alone_and_in_the_mix(world):
    atlas, centres, sv = world
    probe = synthetic.serving_queries(centres, 777, seed=42)
    alone = sv.query(probe)
    others = [synthetic.serving_queries(centres, n, seed=500 + i) for i, n in enumerate([3000, 1, 50, 4000, 900, 12])]
    tickets, lock = [], threading.Lock()

    def submit(x):
        t = sv.submit(x)
        with lock:
            tickets.append(t)

    threads = [threading.Thread(target=submit, args=(x,)) for x in others[:3]]
    for t in threads:
        t.start()
    mine = sv.submit(probe)
    for x in others[3:]:
        submit(x)
    for t in threads:
        t.join()
    mixed = sv.wait(mine)
    for t in tickets:
        sv.wait(t)
    np.testing.assert_array_equal(mixed[0], alone[0])
    np.testing.assert_array_equal(mixed[1], alone[1])
    for a, b in zip(mixed[2], alone[2]):
        np.testing.assert_array_equal(a, b)
    st = sv.stats()
    assert st["requests"] >= 9 and st["batches"] >= 2


def test_bad_requests_are_refused(world):
    _, _, sv = world
    with pytest.raises(ValueError):
        sv.submit(np.zeros((4, 29), np.float32))


@pytest.mark.parametrize("q", [1, 300, 2500, 8192, 10000])
def test_routed_batches_are_exact(built_library, oracle, q):
    """Batches are routed through the atlas ordered once (cells, priority
    tiles, tile balls; each row block's tiles split over column segments that
    share its rows' thresholds): exact all the same, including queries that
    duplicate atlas cells and queries far from every cell."""
    from mrustsc_gb300 import serving

    atlas, centres = synthetic.serving_atlas(seed=5, m=40_000, d=30, clusters=20)
    x = synthetic.serving_queries(centres, q, seed=q)
    dup = min(40, q)
    x[:dup] = atlas[np.arange(dup) * 997]        # exact copies of atlas cells
    if q > 48:
        x[40:48] = 50.0 + np.arange(8)[:, None]  # far from every cell
    with serving.Server(atlas, K, slots=1, max_batch_cells=65536) as sv:
        idx, dist, (indptr, cols, vals), _ = sv.query(x)
    oi, od, _ = oracle.knn_fp64_cross_c(x, atlas, K)
    np.testing.assert_array_equal(idx, oi)
    rel = np.abs(dist.astype(np.float64) - od) / np.maximum(od, 1e-30)
    assert rel.max() <= 1e-6
    assert np.all(dist[:dup, 0] == 0)
    ep, ec, ev = expected_rows(oracle, idx, dist)
    np.testing.assert_array_equal(indptr, ep)
    np.testing.assert_array_equal(cols, ec)
    np.testing.assert_allclose(vals, ev, atol=1e-5, rtol=0)
