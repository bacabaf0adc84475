"""Drop-in for the neighbours half of the reference's extension module
``scrust._scrust`` (crates/scrust-py/src/embedding.rs:60-100, lib.rs:37-40).

Same names, argument meaning, dtypes, return tuples and exceptions:

* ``knn(embedding, k, device) -> (indices u32 (n, k), distances f32 (n, k))``
* ``connectivities(indices, distances) -> (indptr u32, indices u32, values f32, n_cols)``
* ``gpu_available() -> bool``

plus ``smooth_knn_distances(distances) -> (sigmas, rhos)`` for the
per-row bandwidths (crates/scrust-core/src/neighbors.rs:239).

Devices: ``"auto"``, ``"gpu"`` and ``"cuda"`` run the CUDA library.  This
backend has no CPU implementation: ``"cpu"`` raises ``ValueError`` (the
reference's own CPU path serves it), and when no sm_103a GPU is present the
call raises ``RuntimeError`` rather than falling back.  ``"metal"`` raises
``RuntimeError`` as the reference does on a machine without Metal.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib

DEVICES = ("auto", "gpu", "cuda", "cpu", "metal")


def gpu_available() -> bool:
    try:
        return _lib.gpu_available()
    except ImportError:
        return False


def _device_index(device: str) -> int:
    if not isinstance(device, str):
        raise TypeError(f"device must be a str, got {type(device).__name__}")
    if device in ("auto", "gpu", "cuda"):
        return 0
    if device.startswith("cuda:") and device[5:].isdigit():
        return int(device[5:])
    if device == "cpu":
        raise ValueError(
            "device 'cpu' is served by the reference's own CPU path; this backend runs on CUDA devices only"
        )
    if device == "metal":
        raise _lib.ScrustError(_lib.NO_GPU, "no Metal device is available on this machine")
    raise ValueError(f"device must be one of auto, gpu, cuda, cpu, got {device}")


def _array2(obj, dtype, name: str) -> np.ndarray:
    """2-D array of exactly `dtype`; strided views are copied (convert.rs:70-93)."""
    if not isinstance(obj, np.ndarray) or obj.ndim != 2 or obj.dtype != dtype:
        raise ValueError(f"{name} must be a 2-D numpy array of {np.dtype(dtype)}")
    return np.ascontiguousarray(obj)


def _k(k) -> int:
    k = int(k)
    if k < 0:
        raise OverflowError("can't convert negative int to unsigned")
    return k


def knn(embedding, k, device, *, metric: str = "euclidean", form: str = "auto", mode: str = "exact",
        precision: str = "fp16", ordering: str = "auto", list_capacity: int = 0, segments: int = 0):
    """Exact k nearest neighbours, self excluded, nearest first, ties to the smaller id.

    `ordering` ("auto", "off", "on") controls the tensor form's row ordering;
    `list_capacity` and `segments` (0 = automatic) the candidate lists.  They
    change the speed and never the result.
    """
    x = _array2(embedding, np.float32, "embedding")
    k = _k(k)
    dev = _device_index(device)
    n, d = x.shape
    L = _lib.lib()
    st = _lib.Status()
    opts = _lib.options(form=form, metric=metric, mode=mode, precision=precision, ordering=ordering,
                        list_capacity=list_capacity, segments=segments)
    ctx = None
    # Argument errors are reported before a device is required, as the
    # reference validates before dispatching (neighbors.rs:41-57).
    if n and d and k and k < n and k <= 128:
        ctx = _lib.context(dev)
    idx = np.empty((n, k), dtype=np.uint32)
    dist = np.empty((n, k), dtype=np.float32)
    rc = L.scrust_cuda_knn(ctx, _lib.ptr(x) if x.size else None, n, d, k, ctypes.byref(opts),
                           _lib.ptr(idx) if idx.size else None, _lib.ptr(dist) if dist.size else None,
                           ctypes.byref(st))
    _lib.check(rc, st)
    return idx, dist


def connectivities(indices, distances):
    """UMAP fuzzy simplicial set of a kNN graph as CSR parts."""
    idx = _array2(indices, np.uint32, "indices")
    dist = _array2(distances, np.float32, "distances")
    if idx.shape != dist.shape:
        raise _lib.ScrustValueError(_lib.SHAPE, f"expected distances shaped {idx.shape}, got {dist.shape}")
    n, k = idx.shape
    L = _lib.lib()
    st = _lib.Status()
    ctx = _lib.context(0) if n and k else None
    out = ctypes.c_void_p()
    rc = L.scrust_cuda_connectivities(ctx, _lib.ptr(idx) if idx.size else None,
                                      _lib.ptr(dist) if dist.size else None, n, k, ctypes.byref(out),
                                      ctypes.byref(st))
    _lib.check(rc, st)
    return _lib.csr_host_arrays(out)


def smooth_knn_distances(distances):
    """(sigmas f32 (n,), rhos f32 (n,)) of umap's smooth_knn_dist."""
    dist = _array2(distances, np.float32, "distances")
    n, k = dist.shape
    L = _lib.lib()
    st = _lib.Status()
    ctx = _lib.context(0) if n and k else None
    sig = np.empty(n, dtype=np.float32)
    rho = np.empty(n, dtype=np.float32)
    rc = L.scrust_cuda_smooth_knn_distances(ctx, _lib.ptr(dist) if dist.size else None, n, k,
                                            _lib.ptr(sig) if n else None, _lib.ptr(rho) if n else None,
                                            ctypes.byref(st))
    _lib.check(rc, st)
    return sig, rho


def neighbors_graph(embedding, k, device="auto", *, metric: str = "euclidean", form: str = "auto",
                    mode: str = "exact", precision: str = "fp16"):
    """kNN and connectivities in one device pass: (indices, distances, (indptr, cols, vals, n))."""
    x = _array2(embedding, np.float32, "embedding")
    k = _k(k)
    dev = _device_index(device)
    n, d = x.shape
    L = _lib.lib()
    st = _lib.Status()
    opts = _lib.options(form=form, metric=metric, mode=mode, precision=precision)
    ctx = _lib.context(dev) if (n and d and k and k < n and k <= 128) else None
    idx = np.empty((n, k), dtype=np.uint32)
    dist = np.empty((n, k), dtype=np.float32)
    out = ctypes.c_void_p()
    rc = L.scrust_cuda_neighbors_graph(ctx, _lib.ptr(x) if x.size else None, n, d, k, ctypes.byref(opts),
                                       _lib.ptr(idx) if idx.size else None,
                                       _lib.ptr(dist) if dist.size else None, ctypes.byref(out),
                                       ctypes.byref(st))
    _lib.check(rc, st)
    return idx, dist, _lib.csr_host_arrays(out)


def knn_batch(embeddings, k, device, *, metric: str = "euclidean", precision: str = "fp16",
              list_capacity: int = 0):
    """Exact kNN of several independent samples in one tensor-form sweep.

    `embeddings` is a sequence of (n_s, d) f32 arrays with the same d.  Returns
    one (indices, distances) pair per sample, ids local to the sample; each is
    bit-identical to `knn(embeddings[s], k, device, form="tensor")`.
    """
    mats = [_array2(e, np.float32, "embedding") for e in embeddings]
    if not mats:
        raise _lib.ScrustValueError(_lib.SHAPE, "expected at least one sample")
    d = mats[0].shape[1]
    if any(m.shape[1] != d for m in mats):
        raise _lib.ScrustValueError(_lib.SHAPE, "expected every sample to have the same number of dimensions")
    k = _k(k)
    dev = _device_index(device)
    offsets = np.zeros(len(mats) + 1, dtype=np.uint64)
    offsets[1:] = np.cumsum([m.shape[0] for m in mats])
    x = np.ascontiguousarray(np.concatenate(mats, axis=0)) if len(mats) > 1 else mats[0]
    n = int(offsets[-1])
    L = _lib.lib()
    st = _lib.Status()
    opts = _lib.options(form="tensor", metric=metric, precision=precision, list_capacity=list_capacity)
    # Argument errors are reported before a device is required.
    valid = 0 < d <= 61 and 0 < k <= 128 and all(m.shape[0] > k for m in mats)
    ctx = _lib.context(dev) if valid else None
    idx = np.empty((n, k), dtype=np.uint32)
    dist = np.empty((n, k), dtype=np.float32)
    rc = L.scrust_cuda_knn_batch(ctx, _lib.ptr(x) if x.size else None, _lib.ptr(offsets), len(mats), d, k,
                                 ctypes.byref(opts), _lib.ptr(idx) if idx.size else None,
                                 _lib.ptr(dist) if dist.size else None, ctypes.byref(st))
    _lib.check(rc, st)
    return [(idx[int(offsets[s]):int(offsets[s + 1])], dist[int(offsets[s]):int(offsets[s + 1])])
            for s in range(len(mats))]


def neighbors_graph_batch(embeddings, k, device="auto", *, metric: str = "euclidean", precision: str = "fp16",
                          list_capacity: int = 0):
    """kNN and UMAP connectivities of several independent samples in one pass.

    Returns one (indices, distances, (indptr, cols, vals, n)) per sample, ids
    and columns local to the sample; each equals `neighbors_graph` of that
    sample alone with the tensor form.  No reference counterpart.
    """
    mats = [_array2(e, np.float32, "embedding") for e in embeddings]
    if not mats:
        raise _lib.ScrustValueError(_lib.SHAPE, "expected at least one sample")
    d = mats[0].shape[1]
    if any(m.shape[1] != d for m in mats):
        raise _lib.ScrustValueError(_lib.SHAPE, "expected every sample to have the same number of dimensions")
    k = _k(k)
    dev = _device_index(device)
    offsets = np.zeros(len(mats) + 1, dtype=np.uint64)
    offsets[1:] = np.cumsum([m.shape[0] for m in mats])
    x = np.ascontiguousarray(np.concatenate(mats, axis=0)) if len(mats) > 1 else mats[0]
    n = int(offsets[-1])
    L = _lib.lib()
    st = _lib.Status()
    opts = _lib.options(form="tensor", metric=metric, precision=precision, list_capacity=list_capacity)
    valid = 0 < d <= 61 and 0 < k <= 128 and all(m.shape[0] > k for m in mats)
    ctx = _lib.context(dev) if valid else None
    idx = np.empty((n, k), dtype=np.uint32)
    dist = np.empty((n, k), dtype=np.float32)
    out = ctypes.c_void_p()
    rc = L.scrust_cuda_neighbors_graph_batch(ctx, _lib.ptr(x) if x.size else None, _lib.ptr(offsets), len(mats), d, k,
                                             ctypes.byref(opts), _lib.ptr(idx) if idx.size else None,
                                             _lib.ptr(dist) if dist.size else None, ctypes.byref(out),
                                             ctypes.byref(st))
    _lib.check(rc, st)
    indptr, cols, vals, _ = _lib.csr_host_arrays(out)
    return split_batch_graph(offsets, idx, dist, indptr, cols, vals)


def split_batch_graph(offsets, idx, dist, indptr, cols, vals):
    """Per-sample (indices, distances, (indptr, cols, vals, n)) of a batch graph
    laid out as scrust_cuda_neighbors_graph_batch returns it."""
    res = []
    for s in range(len(offsets) - 1):
        a, b = int(offsets[s]), int(offsets[s + 1])
        p0, p1 = int(indptr[a]), int(indptr[b])
        res.append((idx[a:b], dist[a:b], ((indptr[a:b + 1] - indptr[a]).astype(np.uint32), cols[p0:p1],
                                          vals[p0:p1], b - a)))
    return res


def _array1(obj, dtype, name: str) -> np.ndarray:
    if not isinstance(obj, np.ndarray) or obj.ndim != 1 or obj.dtype != dtype:
        raise ValueError(f"{name} must be a 1-D numpy array of {np.dtype(dtype)}")
    return np.ascontiguousarray(obj)


def umap(indptr, indices, values, n_cols, n_components, n_epochs, min_dist, spread, learning_rate,
         negative_sample_rate, seed, device):
    """UMAP layout of a CSR graph: (n, n_components) f32.  The reference's
    signature (crates/scrust-py/src/embedding.rs:102-134); deterministic on
    the GPU (the same bits on every run)."""
    ip = _array1(indptr, np.uint32, "indptr")
    ix = _array1(indices, np.uint32, "indices")
    vl = _array1(values, np.float32, "values")
    for name, v in (("n_cols", n_cols), ("n_components", n_components), ("n_epochs", n_epochs),
                    ("negative_sample_rate", negative_sample_rate), ("seed", seed)):
        if int(v) < 0:
            raise OverflowError(f"can't convert negative int to unsigned ({name})")
    dev = _device_index(device)
    n = len(ip) - 1
    if n < 0 or (n >= 0 and len(ix) != (int(ip[-1]) if n >= 0 and len(ip) else 0)) or len(vl) != len(ix):
        raise _lib.ScrustValueError(_lib.SHAPE, "expected indptr of n + 1 entries ending at len(indices) == len(values)")
    L = _lib.lib()
    p = _lib.UmapParams()
    L.scrust_umap_params_default(ctypes.byref(p))
    p.n_components = int(n_components)
    p.n_epochs = int(n_epochs)
    p.min_dist = float(min_dist)
    p.spread = float(spread)
    p.learning_rate = float(learning_rate)
    p.negative_sample_rate = int(negative_sample_rate)
    p.seed = int(seed)
    out = np.empty((max(n, 0), int(n_components)), dtype=np.float32)
    st = _lib.Status()
    valid = n > 0 and len(ix) > 0 and int(n_components) > 0 and int(n_epochs) > 0
    ctx = _lib.context(dev) if valid else None
    rc = L.scrust_cuda_umap(ctx, _lib.ptr(ip), _lib.ptr(ix) if ix.size else None, _lib.ptr(vl) if vl.size else None,
                            max(n, 0), int(n_cols), ctypes.byref(p), _lib.ptr(out) if out.size else None,
                            ctypes.byref(st))
    _lib.check(rc, st)
    return out


def pca(indptr, indices, values, n_cols, n_components, zero_center, seed, device):
    """Truncated PCA of a cells x genes CSR matrix: a dict of `embedding`
    (n, k), `components` (k, n_genes), `explained_variance` and
    `explained_variance_ratio` (k,), as the reference's binding returns
    (crates/scrust-py/src/preprocess.rs:154-185).  Deterministic on the GPU."""
    ip = _array1(indptr, np.uint32, "indptr")
    ix = _array1(indices, np.uint32, "indices")
    vl = _array1(values, np.float32, "values")
    for name, v in (("n_cols", n_cols), ("n_components", n_components), ("seed", seed)):
        if int(v) < 0:
            raise OverflowError(f"can't convert negative int to unsigned ({name})")
    dev = _device_index(device)
    n = len(ip) - 1
    if n < 0 or len(ix) != int(ip[-1]) or len(vl) != len(ix):
        raise _lib.ScrustValueError(_lib.SHAPE, "expected indptr of n + 1 entries ending at len(indices) == len(values)")
    g, k = int(n_cols), int(n_components)
    L = _lib.lib()
    st = _lib.Status()
    emb = np.empty((n, k), np.float32)
    comps = np.empty((k, g), np.float32)
    var = np.empty(k, np.float32)
    ratio = np.empty(k, np.float32)
    valid = 0 < k <= min(n, g) and n >= 2
    ctx = _lib.context(dev) if valid else None
    rc = L.scrust_cuda_pca(ctx, _lib.ptr(ip), _lib.ptr(ix) if ix.size else None, _lib.ptr(vl) if vl.size else None,
                           n, g, k, 1 if zero_center else 0, int(seed), _lib.ptr(emb) if emb.size else None,
                           _lib.ptr(comps) if comps.size else None, _lib.ptr(var) if var.size else None,
                           _lib.ptr(ratio) if ratio.size else None, ctypes.byref(st))
    _lib.check(rc, st)
    return {"embedding": emb, "components": comps, "explained_variance": var, "explained_variance_ratio": ratio}


def _graph_args(indptr, indices, values, n_cols):
    ip = _array1(indptr, np.uint32, "indptr")
    ix = _array1(indices, np.uint32, "indices")
    vl = _array1(values, np.float32, "values")
    if int(n_cols) < 0:
        raise OverflowError("can't convert negative int to unsigned (n_cols)")
    n = len(ip) - 1
    if n < 0 or len(ix) != int(ip[-1]) or len(vl) != len(ix):
        raise _lib.ScrustValueError(_lib.SHAPE, "expected indptr of n + 1 entries ending at len(indices) == len(values)")
    return ip, ix, vl, n, int(n_cols)


def _cluster(entry, indptr, indices, values, n_cols, resolution, extra, device):
    ip, ix, vl, n, nc = _graph_args(indptr, indices, values, n_cols)
    dev = _device_index(device)
    L = _lib.lib()
    st = _lib.Status()
    labels = np.empty(max(n, 0), np.uint32)
    q = ctypes.c_double(0.0)
    count = ctypes.c_uint64(0)
    # Argument errors come before a device is required, as in the reference.
    valid = n > 0 and nc == n and math.isfinite(float(resolution)) and float(resolution) > 0
    ctx = _lib.context(dev) if valid else None
    rc = getattr(L, entry)(ctx, _lib.ptr(ip), _lib.ptr(ix) if ix.size else None, _lib.ptr(vl) if vl.size else None,
                           max(n, 0), nc, float(resolution), *extra, _lib.ptr(labels) if labels.size else None,
                           ctypes.byref(q), ctypes.byref(count), ctypes.byref(st))
    _lib.check(rc, st)
    return labels, float(q.value), int(count.value)


def leiden(indptr, indices, values, n_cols, resolution, n_iterations, seed, device):
    """Leiden communities of a square CSR graph: (labels u32, modularity,
    n_communities), labels numbered by descending community size.  The
    reference's signature (crates/scrust-py/src/cluster.rs:30-49); the moves
    run in parallel rounds on the GPU, deterministic for a seed."""
    for name, v in (("n_iterations", n_iterations), ("seed", seed)):
        if int(v) < 0:
            raise OverflowError(f"can't convert negative int to unsigned ({name})")
    return _cluster("scrust_cuda_leiden", indptr, indices, values, n_cols, resolution,
                    (int(n_iterations), int(seed)), device)


def louvain(indptr, indices, values, n_cols, resolution, seed, device):
    """Louvain communities (crates/scrust-py/src/cluster.rs:51-69), as leiden."""
    if int(seed) < 0:
        raise OverflowError("can't convert negative int to unsigned (seed)")
    return _cluster("scrust_cuda_louvain", indptr, indices, values, n_cols, resolution, (int(seed),), device)


def modularity(indptr, indices, values, n_cols, labels, resolution):
    """Modularity of `labels` on the graph (crates/scrust-py/src/cluster.rs:71-86),
    computed on the GPU."""
    ip, ix, vl, n, nc = _graph_args(indptr, indices, values, n_cols)
    lab = _array1(labels, np.uint32, "labels")
    L = _lib.lib()
    st = _lib.Status()
    q = ctypes.c_double(0.0)
    valid = n > 0 and nc == n and len(lab) == n and math.isfinite(float(resolution)) and float(resolution) > 0
    ctx = _lib.context(0) if valid else None
    rc = L.scrust_cuda_modularity(ctx, _lib.ptr(ip), _lib.ptr(ix) if ix.size else None,
                                  _lib.ptr(vl) if vl.size else None, max(n, 0), nc,
                                  _lib.ptr(lab) if lab.size else None, len(lab), float(resolution), ctypes.byref(q),
                                  ctypes.byref(st))
    _lib.check(rc, st)
    return float(q.value)
