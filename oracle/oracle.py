"""The oracle for the pp.neighbors path -- TEST INFRASTRUCTURE ONLY.

ctypes access to ``neighbors_oracle.c`` (a C restatement of the reference's
CPU path, the CPU twin of its Metal kernel, and the FP64 exact kNN).  Only the
tests, the smoke entry point and bench.py's CPU-baseline leg import this
module, and only as the checker or as the timed CPU baseline.  The shipped
library never imports it.

Functions mirror the reference files they restate:
  knn_reference_cpu  crates/scrust-core/src/neighbors.rs:29-101, 171-191
  ExpansionCPU       the same with the tile product on a BLAS SGEMM
  knn_metal_twin     crates/scrust-gpu/src/kernels/knn.rs:135-158, 282-313
  knn_fp64           tests/test_neighbors_audit.py:52-61
  knn_fp64_cross_c   the same for query rows against reference rows
  smooth_knn         crates/scrust-core/src/neighbors.rs:239-298
  connectivities     crates/scrust-core/src/neighbors.rs:208-372
  umap, fit_ab_params, tau_words   crates/scrust-core/src/umap.rs:64-509 (umap_oracle.c)
  leiden, louvain, modularity      crates/scrust-core/src/cluster.rs:88-850 (cluster_oracle.c)
"""

from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess
import threading

import numpy as np

_HERE = pathlib.Path(__file__).resolve().parent
_SRC = _HERE / "neighbors_oracle.c"
_SOURCES = (_SRC, _HERE / "umap_oracle.c", _HERE / "cluster_oracle.c")
_OUT = _HERE / "_build" / "liboracle.so"
_LOCK = threading.Lock()
_LIB = None

OK, SHAPE, INVALID_PARAMETER, OOM = 0, 1, 2, 6


class OracleError(ValueError):
    """An argument the reference would reject (Shape / InvalidParameter)."""


def build(force: bool = False) -> pathlib.Path:
    """Compile the restatement with gcc (no -march flags: same code on x86 and Arm)."""
    _OUT.parent.mkdir(parents=True, exist_ok=True)
    newest = max(src.stat().st_mtime for src in _SOURCES)
    if force or not _OUT.exists() or _OUT.stat().st_mtime < newest:
        tmp = _OUT.with_suffix(f".{os.getpid()}.tmp.so")
        cmd = [
            "gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
            *map(str, _SOURCES), "-o", str(tmp), "-lm",
        ]
        subprocess.run(cmd, check=True)
        os.replace(tmp, _OUT)
    return _OUT


def _lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            lib = ctypes.CDLL(str(build()))
            i64, f32p, u32p, f64p, i64p = (
                ctypes.c_int64,
                ctypes.POINTER(ctypes.c_float),
                ctypes.POINTER(ctypes.c_uint32),
                ctypes.POINTER(ctypes.c_double),
                ctypes.POINTER(ctypes.c_int64),
            )
            lib.oracle_knn_reference_cpu.argtypes = [f32p, i64, i64, i64, i64, u32p, f32p]
            lib.oracle_knn_reference_cpu_rows.argtypes = [f32p, i64, i64, i64, i64p, i64, u32p, f32p]
            lib.oracle_knn_metal_twin.argtypes = [f32p, i64, i64, i64, u32p, f32p]
            lib.oracle_knn_fp64_rows.argtypes = [f32p, i64, i64, i64, i64p, i64, u32p, f64p, f32p]
            lib.oracle_knn_cosine_fp64_rows.argtypes = [f32p, i64, i64, i64, i64p, i64, u32p, f64p, f32p]
            lib.oracle_knn_fp64_cross.argtypes = [f32p, i64, f32p, i64, i64, i64, u32p, f64p, f32p]
            lib.oracle_centred_norms.argtypes = [f32p, i64, i64, f32p, f32p]
            lib.oracle_expansion_select.argtypes = [f32p, i64, i64, i64, i64p, f32p, i64, u32p, f32p]
            lib.oracle_smooth_knn.argtypes = [f32p, i64, i64, f32p, f32p]
            lib.oracle_connectivities.argtypes = [u32p, f32p, i64, i64, u32p, u32p, f32p, i64p]
            lib.oracle_directed_weights.argtypes = [u32p, f32p, i64, i64, f32p]
            lib.oracle_centred.argtypes = [f32p, i64, i64, f32p]
            lib.oracle_unrolled_sum_f32.argtypes = [f32p, i64]
            lib.oracle_unrolled_sum_f32.restype = ctypes.c_float
            lib.oracle_num_threads.restype = ctypes.c_int
            lib.oracle_tau_words.argtypes = [ctypes.c_uint64, i64, u32p]
            lib.oracle_leiden.argtypes = [u32p, u32p, f32p, i64, i64, ctypes.c_double, i64, ctypes.c_uint64, u32p,
                                          f64p, i64p]
            lib.oracle_louvain.argtypes = [u32p, u32p, f32p, i64, i64, ctypes.c_double, ctypes.c_uint64, u32p, f64p,
                                           i64p]
            lib.oracle_modularity.argtypes = [u32p, u32p, f32p, i64, i64, u32p, i64, ctypes.c_double, f64p]
            lib.oracle_fit_ab_params.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.POINTER(ctypes.c_float),
                                                 ctypes.POINTER(ctypes.c_float)]
            lib.oracle_umap.argtypes = [u32p, u32p, f32p, i64, i64, i64, i64, ctypes.c_float, ctypes.c_float,
                                        ctypes.c_float, i64, ctypes.c_uint64, f32p]
            _LIB = lib
    return _LIB


def _p(array, ctype):
    return array.ctypes.data_as(ctypes.POINTER(ctype))


def _check(rc: int, what: str) -> None:
    if rc == SHAPE:
        raise OracleError(f"{what}: shape")
    if rc == INVALID_PARAMETER:
        raise OracleError(f"{what}: invalid parameter")
    if rc != OK:
        raise MemoryError(f"{what}: status {rc}")


def _f32(x) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.float32)


def num_threads() -> int:
    return int(_lib().oracle_num_threads())


def knn_reference_cpu(x, k: int, tile_rows: int = 0):
    """The reference CPU kNN (expansion form, snap, (d^2, id) order)."""
    x = _f32(x)
    n, d = x.shape if x.ndim == 2 else (0, 0)
    idx = np.zeros((max(n, 1), max(k, 1)), np.uint32)
    dist = np.zeros((max(n, 1), max(k, 1)), np.float32)
    _check(_lib().oracle_knn_reference_cpu(_p(x, ctypes.c_float), n, d, k, tile_rows,
                                           _p(idx, ctypes.c_uint32), _p(dist, ctypes.c_float)),
           "knn_reference_cpu")
    return idx[:n, :k], dist[:n, :k]


def knn_reference_cpu_rows(x, k: int, rows):
    """The reference CPU kNN for the query rows `rows`, each against all cells."""
    x = _f32(x)
    n, d = x.shape
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    idx = np.zeros((len(rows), k), np.uint32)
    dist = np.zeros((len(rows), k), np.float32)
    _check(_lib().oracle_knn_reference_cpu_rows(_p(x, ctypes.c_float), n, d, k,
                                                _p(rows, ctypes.c_int64), len(rows),
                                                _p(idx, ctypes.c_uint32), _p(dist, ctypes.c_float)),
           "knn_reference_cpu_rows")
    return idx, dist


class ExpansionCPU:
    """The reference CPU kNN (neighbors.rs:29-101) with its tile product on a
    BLAS, as candle runs it: centred coordinates and squared norms are made
    once (the setup of knn_tiled), then each tile of query rows is one SGEMM
    (numpy's BLAS, all host threads) followed by the affine, snap and
    selection in C (all host threads).  Used to time the reference's CPU path
    on a sample of query rows; tiles are MAX_TILE_ELEMENTS = 64 Mi wide as in
    neighbors.rs:30."""

    TILE_ELEMENTS = 64 * 1024 * 1024

    def __init__(self, x):
        x = _f32(x)
        self.n, self.d = x.shape
        self.c = np.zeros_like(x)
        self.sq = np.zeros(self.n, np.float32)
        _check(_lib().oracle_centred_norms(_p(x, ctypes.c_float), self.n, self.d, _p(self.c, ctypes.c_float),
                                           _p(self.sq, ctypes.c_float)), "centred_norms")
        self.ct = np.ascontiguousarray(self.c.T)
        self.tile_rows = max(1, self.TILE_ELEMENTS // max(1, self.n))

    def knn_rows(self, k: int, rows):
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        idx = np.zeros((len(rows), k), np.uint32)
        dist = np.zeros((len(rows), k), np.float32)
        for a in range(0, len(rows), self.tile_rows):
            r = rows[a:a + self.tile_rows]
            g = np.ascontiguousarray(self.c[r] @ self.ct, dtype=np.float32)
            _check(_lib().oracle_expansion_select(_p(g, ctypes.c_float), len(r), self.n, self.d,
                                                  _p(r, ctypes.c_int64), _p(self.sq, ctypes.c_float), k,
                                                  _p(idx[a:], ctypes.c_uint32), _p(dist[a:], ctypes.c_float)),
                   "expansion_select")
        return idx, dist


def knn_metal_twin(x, k: int):
    """CPU twin of the reference Metal kernel (difference form on centred data + snap)."""
    x = _f32(x)
    n, d = x.shape if x.ndim == 2 else (0, 0)
    idx = np.zeros((max(n, 1), max(k, 1)), np.uint32)
    dist = np.zeros((max(n, 1), max(k, 1)), np.float32)
    _check(_lib().oracle_knn_metal_twin(_p(x, ctypes.c_float), n, d, k,
                                        _p(idx, ctypes.c_uint32), _p(dist, ctypes.c_float)),
           "knn_metal_twin")
    return idx[:n, :k], dist[:n, :k]


def knn_fp64(x, k: int, rows=None, metric: str = "euclidean"):
    """FP64 exact kNN: (idx u32, d64 f64, dist f32) for `rows` (default all)."""
    x = _f32(x)
    n, d = x.shape
    if rows is None:
        nrows, rows_p = n, None
    else:
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        nrows, rows_p = len(rows), _p(rows, ctypes.c_int64)
    idx = np.zeros((nrows, k), np.uint32)
    d64 = np.zeros((nrows, k), np.float64)
    dist = np.zeros((nrows, k), np.float32)
    fn = _lib().oracle_knn_fp64_rows if metric == "euclidean" else _lib().oracle_knn_cosine_fp64_rows
    _check(fn(_p(x, ctypes.c_float), n, d, k, rows_p, nrows, _p(idx, ctypes.c_uint32),
              _p(d64, ctypes.c_double), _p(dist, ctypes.c_float)), "knn_fp64")
    return idx, d64, dist


def smooth_knn(distances):
    dist = _f32(distances)
    n, k = dist.shape
    sig = np.zeros(n, np.float32)
    rho = np.zeros(n, np.float32)
    _check(_lib().oracle_smooth_knn(_p(dist, ctypes.c_float), n, k, _p(sig, ctypes.c_float),
                                    _p(rho, ctypes.c_float)), "smooth_knn")
    return sig, rho


def directed_weights(indices, distances):
    idx = np.ascontiguousarray(indices, dtype=np.uint32)
    dist = _f32(distances)
    n, k = dist.shape
    w = np.zeros((n, k), np.float32)
    _check(_lib().oracle_directed_weights(_p(idx, ctypes.c_uint32), _p(dist, ctypes.c_float), n, k,
                                          _p(w, ctypes.c_float)), "directed_weights")
    return w


def connectivities(indices, distances):
    """(indptr u32, indices u32, values f32, n_cols), the reference's return shape."""
    idx = np.ascontiguousarray(indices, dtype=np.uint32)
    dist = _f32(distances)
    if idx.shape != dist.shape or idx.ndim != 2:
        raise OracleError("connectivities: shape")
    n, k = dist.shape
    indptr = np.zeros(n + 1, np.uint32)
    cols = np.zeros(max(2 * n * k, 1), np.uint32)
    vals = np.zeros(max(2 * n * k, 1), np.float32)
    nnz = np.zeros(1, np.int64)
    _check(_lib().oracle_connectivities(_p(idx, ctypes.c_uint32), _p(dist, ctypes.c_float), n, k,
                                        _p(indptr, ctypes.c_uint32), _p(cols, ctypes.c_uint32),
                                        _p(vals, ctypes.c_float), _p(nnz, ctypes.c_int64)),
           "connectivities")
    m = int(nnz[0])
    return indptr, cols[:m].copy(), vals[:m].copy(), n


def centred(x):
    x = _f32(x)
    out = np.zeros_like(x)
    _check(_lib().oracle_centred(_p(x, ctypes.c_float), x.shape[0], x.shape[1],
                                 _p(out, ctypes.c_float)), "centred")
    return out


def unrolled_sum(x) -> np.float32:
    x = _f32(np.ravel(x))
    return np.float32(_lib().oracle_unrolled_sum_f32(_p(x, ctypes.c_float), x.size))


def exact_knn_numpy(x, k: int):
    """tests/test_neighbors_audit.py:52-61 verbatim in semantics (numpy, small n only)."""
    x64 = np.asarray(x, dtype=np.float64)
    d = np.sqrt(np.maximum(((x64[:, None, :] - x64[None, :, :]) ** 2).sum(-1), 0.0))
    n = d.shape[0]
    indices = np.zeros((n, k), dtype=np.int64)
    for cell in range(n):
        order = sorted((j for j in range(n) if j != cell), key=lambda j: (d[cell, j], j))
        indices[cell] = order[:k]
    return indices, np.take_along_axis(d, indices, 1)


def knn_fp64_cross_c(queries, reference, k: int):
    """Exact k nearest reference rows of every query row in FP64 (the C
    restatement, any size): (idx u32, d64 f64, dist f32), the semantics of
    tests/test_neighbors_audit.py:52-61 for a query-versus-reference solve
    with no self-exclusion and the lowest reference index on ties."""
    q = _f32(queries)
    r = _f32(reference)
    nq, d = q.shape
    idx = np.zeros((nq, k), np.uint32)
    d64 = np.zeros((nq, k), np.float64)
    dist = np.zeros((nq, k), np.float32)
    _check(_lib().oracle_knn_fp64_cross(_p(q, ctypes.c_float), nq, _p(r, ctypes.c_float), r.shape[0], d, k,
                                        _p(idx, ctypes.c_uint32), _p(d64, ctypes.c_double),
                                        _p(dist, ctypes.c_float)), "knn_fp64_cross")
    return idx, d64, dist


def knn_fp64_cross(queries, reference, k: int):
    """Exact k nearest reference rows of every query row in FP64 (difference
    form, lowest reference index on ties, no self-exclusion): the semantics of
    tests/test_neighbors_audit.py:52-61 for a query-versus-reference solve.
    numpy; returns (indices, FP64 distances)."""
    q64 = np.asarray(queries, dtype=np.float64)
    r64 = np.asarray(reference, dtype=np.float64)
    idx = np.zeros((len(q64), k), dtype=np.int64)
    dist = np.zeros((len(q64), k), dtype=np.float64)
    for b in range(0, len(q64), 256):
        qb = q64[b:b + 256]
        d2 = ((qb[:, None, :] - r64[None, :, :]) ** 2).sum(-1)
        order = np.lexsort((np.broadcast_to(np.arange(len(r64)), d2.shape), d2), axis=1)[:, :k]
        idx[b:b + 256] = order
        dist[b:b + 256] = np.sqrt(np.take_along_axis(d2, order, 1))
    return idx, dist


def tau_words(seed: int, count: int) -> np.ndarray:
    """The first words of the reference's TauRng::new(seed) (umap.rs:174-229)."""
    out = np.zeros(count, np.uint32)
    _lib().oracle_tau_words(ctypes.c_uint64(seed), count, _p(out, ctypes.c_uint32))
    return out


def fit_ab_params(min_dist: float, spread: float) -> tuple[float, float]:
    a, b = ctypes.c_float(), ctypes.c_float()
    _check(_lib().oracle_fit_ab_params(min_dist, spread, ctypes.byref(a), ctypes.byref(b)), "fit_ab_params")
    return a.value, b.value


def umap(indptr, indices, values, n_cols: int, n_components: int = 2, n_epochs: int = 200, min_dist: float = 0.5,
         spread: float = 1.0, learning_rate: float = 1.0, negative_sample_rate: int = 5, seed: int = 0):
    """The reference's CPU UMAP layout (umap.rs:64), (n, n_components) f32."""
    ip = np.ascontiguousarray(indptr, dtype=np.uint32)
    ix = np.ascontiguousarray(indices, dtype=np.uint32)
    vl = _f32(values)
    n = len(ip) - 1
    out = np.zeros((max(n, 1), max(n_components, 1)), np.float32)
    _check(_lib().oracle_umap(_p(ip, ctypes.c_uint32), _p(ix, ctypes.c_uint32), _p(vl, ctypes.c_float), n, n_cols,
                              n_components, n_epochs, min_dist, spread, learning_rate, negative_sample_rate,
                              ctypes.c_uint64(seed), _p(out, ctypes.c_float)), "umap")
    return out[:n, :n_components]


def _csr32(indptr, indices, values):
    return (np.ascontiguousarray(indptr, dtype=np.uint32), np.ascontiguousarray(indices, dtype=np.uint32),
            _f32(values))


def leiden(indptr, indices, values, n_cols: int, resolution: float = 1.0, n_iterations: int = 2, seed: int = 0):
    """(labels u32, modularity, n_communities) of the restated Leiden (cluster.rs:88)."""
    ip, ix, vl = _csr32(indptr, indices, values)
    n = len(ip) - 1
    labels = np.zeros(max(n, 1), np.uint32)
    q = ctypes.c_double()
    nc = np.zeros(1, np.int64)
    _check(_lib().oracle_leiden(_p(ip, ctypes.c_uint32), _p(ix, ctypes.c_uint32), _p(vl, ctypes.c_float), n, n_cols,
                                resolution, n_iterations, ctypes.c_uint64(seed), _p(labels, ctypes.c_uint32),
                                ctypes.byref(q), _p(nc, ctypes.c_int64)), "leiden")
    return labels[:n], q.value, int(nc[0])


def louvain(indptr, indices, values, n_cols: int, resolution: float = 1.0, seed: int = 0):
    """(labels u32, modularity, n_communities) of the restated Louvain (cluster.rs:125)."""
    ip, ix, vl = _csr32(indptr, indices, values)
    n = len(ip) - 1
    labels = np.zeros(max(n, 1), np.uint32)
    q = ctypes.c_double()
    nc = np.zeros(1, np.int64)
    _check(_lib().oracle_louvain(_p(ip, ctypes.c_uint32), _p(ix, ctypes.c_uint32), _p(vl, ctypes.c_float), n, n_cols,
                                 resolution, ctypes.c_uint64(seed), _p(labels, ctypes.c_uint32), ctypes.byref(q),
                                 _p(nc, ctypes.c_int64)), "louvain")
    return labels[:n], q.value, int(nc[0])


def modularity(indptr, indices, values, n_cols: int, labels, resolution: float = 1.0) -> float:
    """Q of a labelling (cluster.rs:148)."""
    ip, ix, vl = _csr32(indptr, indices, values)
    lb = np.ascontiguousarray(labels, dtype=np.uint32)
    q = ctypes.c_double()
    _check(_lib().oracle_modularity(_p(ip, ctypes.c_uint32), _p(ix, ctypes.c_uint32), _p(vl, ctypes.c_float),
                                    len(ip) - 1, n_cols, _p(lb, ctypes.c_uint32), len(lb), resolution,
                                    ctypes.byref(q)), "modularity")
    return q.value
