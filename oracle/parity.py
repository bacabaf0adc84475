"""Parity checks of GPU results against the oracle -- TEST INFRASTRUCTURE ONLY.

The tests and bench.py's parity leg (outside every timed region) use these
helpers to compare what the CUDA library returned with the C restatement in
``neighbors_oracle.c``:

* kNN rows against the FP64 exact kNN (tests/test_neighbors_audit.py:52-61 of
  the reference): neighbour ids bit-exact with the lowest-index tie-break,
  distances within 1e-6 relative (exact zeros stay zero);
* a connectivities CSR against the restatement of
  crates/scrust-core/src/neighbors.rs:208-372 run on the same kNN graph:
  structure bit-exact, values within 1e-5 absolute;
* query rows against a reference (the serving form) with the FP64
  query-versus-reference kNN and the directed weights of those rows.

The rows checked at scale are a seeded random sample plus every row with a
neighbour at distance 0 and every row whose k-th and (k+1)-th neighbours sit
within a relative 1e-5 of each other (found from a k+1 solve).
"""

from __future__ import annotations

import numpy as np

from . import oracle

DIST_RTOL = 1e-6
CONN_ATOL = 1e-5
NEAR_TIE_RTOL = 1e-5


def select_rows(n: int, dist: np.ndarray, dist_k1: np.ndarray | None = None, n_random: int = 10_000,
                seed: int = 0) -> tuple[np.ndarray, dict]:
    """Rows to check: `n_random` seeded random rows, all rows with a
    zero-distance neighbour, and (given a k+1 solve's distances) all rows
    whose k-th and (k+1)-th distances are within NEAR_TIE_RTOL."""
    rng = np.random.default_rng(seed)
    rand = rng.choice(n, size=min(n, n_random), replace=False)
    zero = np.nonzero(dist[:, 0] == 0.0)[0]
    near = np.zeros(0, np.int64)
    if dist_k1 is not None:
        dk = dist_k1[:, -2].astype(np.float64)
        dk1 = dist_k1[:, -1].astype(np.float64)
        near = np.nonzero(dk1 - dk <= NEAR_TIE_RTOL * np.maximum(dk, 1e-30))[0]
    rows = np.unique(np.concatenate([rand, zero, near]).astype(np.int64))
    return rows, {"random": int(len(rand)), "zero_distance": int(len(zero)), "near_tie": int(len(near))}


def knn_rows_report(x: np.ndarray, k: int, idx: np.ndarray, dist: np.ndarray, rows: np.ndarray) -> dict:
    """Compares the GPU rows `rows` of (idx, dist) with the FP64 oracle."""
    oi, od64, _ = oracle.knn_fp64(x, k, rows)
    gi = np.asarray(idx)[rows].astype(np.uint32)
    gd = np.asarray(dist)[rows].astype(np.float64)
    exact = (gi == oi).all(axis=1)
    hits = sum(len(set(a.tolist()) & set(b.tolist())) for a, b in zip(gi, oi))
    zero = od64 == 0
    zeros_ok = bool(np.all(gd[zero] == 0))
    rel = np.abs(gd[~zero] - od64[~zero]) / od64[~zero]
    return {"rows": int(len(rows)), "exact_rows": int(exact.sum()), "recall": hits / (len(rows) * k),
            "max_rel_dist_err": float(rel.max(initial=0.0)), "zero_distances_exact": zeros_ok,
            "first_bad_rows": rows[~exact][:5].tolist()}


def knn_rows_ok(report: dict) -> bool:
    return (report["exact_rows"] == report["rows"] and report["max_rel_dist_err"] <= DIST_RTOL
            and report["zero_distances_exact"])


def connectivities_report(idx: np.ndarray, dist: np.ndarray, csr) -> dict:
    """Compares a CSR (indptr, indices, values[, n]) with the oracle's
    connectivities of the same kNN graph."""
    ref = oracle.connectivities(np.asarray(idx).astype(np.uint32), np.asarray(dist, np.float32))
    indptr, cols, vals = (np.asarray(a) for a in csr[:3])
    same_indptr = bool(np.array_equal(indptr.astype(np.uint32), ref[0]))
    same_cols = same_indptr and bool(np.array_equal(cols.astype(np.uint32), ref[1]))
    err = float(np.abs(vals.astype(np.float64) - ref[2].astype(np.float64)).max(initial=0.0)) if same_cols else None
    return {"nnz": int(len(ref[1])), "nnz_gpu": int(len(cols)), "structure_equal": same_cols,
            "max_abs_err": err}


def connectivities_ok(report: dict) -> bool:
    return report["structure_equal"] and report["max_abs_err"] is not None and report["max_abs_err"] <= CONN_ATOL


def query_rows_expected(idx: np.ndarray, dist: np.ndarray):
    """Directed connectivity rows of query rows (no self to drop; columns
    ascending), from the oracle's smooth_knn and directed weights: the ids are
    shifted past every row index before the oracle sees them, so that no id
    is taken for the row itself."""
    shifted = (np.asarray(idx).astype(np.uint64) + (1 << 31)).astype(np.uint32)
    w = oracle.directed_weights(shifted, dist)
    indptr = [0]
    cols, vals = [], []
    for i in range(len(idx)):
        keep = w[i] != 0
        order = np.argsort(idx[i][keep], kind="stable")
        cols.extend(idx[i][keep][order].tolist())
        vals.extend(w[i][keep][order].tolist())
        indptr.append(len(cols))
    return np.asarray(indptr, np.uint32), np.asarray(cols, np.uint32), np.asarray(vals, np.float32)


def cross_rows_report(queries: np.ndarray, reference: np.ndarray, k: int, idx: np.ndarray,
                      dist: np.ndarray) -> dict:
    """Query rows against the FP64 query-versus-reference oracle."""
    oi, od64, _ = oracle.knn_fp64_cross_c(queries, reference, k)
    gi = np.asarray(idx).astype(np.uint32)
    gd = np.asarray(dist).astype(np.float64)
    exact = (gi == oi).all(axis=1)
    zero = od64 == 0
    rel = np.abs(gd[~zero] - od64[~zero]) / od64[~zero]
    return {"rows": int(len(gi)), "exact_rows": int(exact.sum()), "max_rel_dist_err": float(rel.max(initial=0.0)),
            "zero_distances_exact": bool(np.all(gd[zero] == 0))}
