"""The oracle-side helpers used at the benchmark sizes (CPU only): the BLAS
form of the reference CPU path, the FP64 query-versus-reference kNN, and the
parity reports that the GPU tests and the bench's parity leg build on."""

from __future__ import annotations

import numpy as np

from mrustsc_gb300 import synthetic


def test_blas_expansion_equals_the_sequential_restatement(oracle):
    x = synthetic.plain_small(seed=3)
    engine = oracle.ExpansionCPU(x)
    rows = np.arange(0, len(x), 7)
    idx, dist = engine.knn_rows(15, rows)
    ri, rd = oracle.knn_reference_cpu_rows(x, 15, rows)
    # The SGEMM's summation order is the BLAS's own (the reference's is
    # gemm 0.19's, unpublished): lists agree wherever the expansion does not
    # tie, which on this data is every row.
    np.testing.assert_array_equal(idx, ri)
    np.testing.assert_allclose(dist, rd, rtol=1e-4, atol=1e-3)


def test_cross_knn_matches_numpy(oracle):
    rng = np.random.default_rng(5)
    ref = rng.normal(size=(2000, 9)).astype(np.float32)
    q = rng.normal(size=(40, 9)).astype(np.float32)
    q[0] = ref[3]
    ref[4] = ref[3]
    i, d64, _ = oracle.knn_fp64_cross_c(q, ref, 11)
    ni, nd = oracle.knn_fp64_cross(q, ref, 11)
    np.testing.assert_array_equal(i, ni)
    np.testing.assert_allclose(d64, nd, rtol=1e-12, atol=0)
    assert i[0][:2].tolist() == [3, 4]


def test_parity_reports_accept_the_oracle_and_catch_a_planted_error(oracle):
    from oracle import parity

    x = synthetic.mixture(1500, 20, clusters=5, dup_frac=0.02, seed=9)
    idx, _, dist = oracle.knn_fp64(x, 10)
    _, _, dist11 = oracle.knn_fp64(x, 11)
    rows, kinds = parity.select_rows(len(x), dist, dist11, n_random=200, seed=1)
    assert kinds["zero_distance"] >= 30 and len(rows) >= 200
    rep = parity.knn_rows_report(x, 10, idx, dist, rows)
    assert parity.knn_rows_ok(rep)
    conn = oracle.connectivities(idx, dist)
    assert parity.connectivities_ok(parity.connectivities_report(idx, dist, conn))
    bad = idx.copy()
    r = int(rows[0])
    bad[r, [0, 1]] = bad[r, [1, 0]]
    assert not parity.knn_rows_ok(parity.knn_rows_report(x, 10, bad, dist, rows))
    vals = conn[2].copy()
    vals[0] += 1e-4
    assert not parity.connectivities_ok(parity.connectivities_report(idx, dist, (conn[0], conn[1], vals)))
