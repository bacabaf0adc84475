"""ctypes binding of ``libscrust_cuda.so`` (declared in include/scrust_cuda.h).

The library is built in-tree by :mod:`mrustsc_gb300.build`.  Loading never
falls back to anything: if the library is missing or fails to load, the
caller gets an :class:`ImportError` naming the file.  Status codes map to
exceptions exactly as the reference's PyO3 layer does
(crates/scrust-py/src/lib.rs:26-35): shape and parameter errors raise
``ValueError``, every other error ``RuntimeError``.
"""

from __future__ import annotations

import ctypes
import pathlib
import threading

import numpy as np

LIB_PATH = pathlib.Path(__file__).resolve().parent / "libscrust_cuda.so"

OK, SHAPE, INVALID_PARAMETER, NO_GPU, KERNEL, NOT_CONVERGED, OOM, TIMEOUT = range(8)

FORM_PLAIN, FORM_TENSOR, FORM_AUTO = 0, 1, 2
TENSOR_FORM_READY = True
METRIC_EUCLIDEAN, METRIC_COSINE = 0, 1
MODE_EXACT, MODE_REFERENCE_SNAP = 0, 1
PRECISION_FP16, PRECISION_BF16 = 0, 1

FORMS = {"plain": FORM_PLAIN, "tensor": FORM_TENSOR, "auto": FORM_AUTO}
METRICS = {"euclidean": METRIC_EUCLIDEAN, "cosine": METRIC_COSINE}
MODES = {"exact": MODE_EXACT, "reference_snap": MODE_REFERENCE_SNAP}
PRECISIONS = {"fp16": PRECISION_FP16, "bf16": PRECISION_BF16}
ORDERINGS = {"auto": 0, "off": 1, "on": 2}


class Status(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int32), ("message", ctypes.c_char * 256)]


class KnnOptions(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("form", ctypes.c_int32),
        ("metric", ctypes.c_int32),
        ("mode", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("list_capacity", ctypes.c_uint32),
        ("segments", ctypes.c_uint32),
        ("ordering", ctypes.c_int32),
        ("reserved", ctypes.c_uint32 * 8),
    ]


class UmapParams(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("n_components", ctypes.c_uint32),
        ("n_epochs", ctypes.c_uint32),
        ("min_dist", ctypes.c_float),
        ("spread", ctypes.c_float),
        ("learning_rate", ctypes.c_float),
        ("negative_sample_rate", ctypes.c_uint32),
        ("reserved0", ctypes.c_uint32),
        ("seed", ctypes.c_uint64),
        ("reserved", ctypes.c_uint32 * 8),
    ]


class ScrustError(RuntimeError):
    """A non-parameter failure reported by the CUDA library."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class ScrustValueError(ValueError):
    """SHAPE / INVALID_PARAMETER, as the reference raises ValueError."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


_LOCK = threading.Lock()
_LIB = None
_CONTEXTS: dict[int, int] = {}

# Every entry point the header declares, with its ctypes signature.
_P = ctypes.c_void_p
_SIGNATURES = {
    "scrust_knn_options_default": (None, [ctypes.POINTER(KnnOptions)]),
    "scrust_cuda_gpu_available": (ctypes.c_int32, []),
    "scrust_cuda_context_create": (_P, [ctypes.c_int32, ctypes.POINTER(Status)]),
    "scrust_cuda_context_destroy": (None, [_P]),
    "scrust_cuda_context_stream": (_P, [_P]),
    "scrust_cuda_max_supported_k": (ctypes.c_uint32, [_P]),
    "scrust_cuda_knn": (ctypes.c_int32, [_P, _P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                          ctypes.POINTER(KnnOptions), _P, _P, ctypes.POINTER(Status)]),
    "scrust_cuda_knn_device": (ctypes.c_int32, [_P, _P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                                 ctypes.POINTER(KnnOptions), _P, _P, ctypes.POINTER(Status)]),
    "scrust_cuda_connectivities": (ctypes.c_int32, [_P, _P, _P, ctypes.c_uint64, ctypes.c_uint32,
                                                     ctypes.POINTER(_P), ctypes.POINTER(Status)]),
    "scrust_cuda_connectivities_device": (ctypes.c_int32, [_P, _P, _P, ctypes.c_uint64, ctypes.c_uint32,
                                                            ctypes.POINTER(_P), ctypes.POINTER(Status)]),
    "scrust_cuda_smooth_knn_distances": (ctypes.c_int32, [_P, _P, ctypes.c_uint64, ctypes.c_uint32, _P, _P,
                                                           ctypes.POINTER(Status)]),
    "scrust_cuda_neighbors_graph": (ctypes.c_int32, [_P, _P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                                      ctypes.POINTER(KnnOptions), _P, _P, ctypes.POINTER(_P),
                                                      ctypes.POINTER(Status)]),
    "scrust_cuda_neighbors_graph_device": (ctypes.c_int32, [_P, _P, ctypes.c_uint64, ctypes.c_uint64,
                                                             ctypes.c_uint32, ctypes.POINTER(KnnOptions), _P, _P,
                                                             ctypes.POINTER(_P), ctypes.POINTER(Status)]),
    "scrust_csr_n_rows": (ctypes.c_uint64, [_P]),
    "scrust_csr_n_cols": (ctypes.c_uint64, [_P]),
    "scrust_csr_nnz": (ctypes.c_uint64, [_P]),
    "scrust_csr_on_device": (ctypes.c_int32, [_P]),
    "scrust_csr_indptr": (_P, [_P]),
    "scrust_csr_indices": (_P, [_P]),
    "scrust_csr_values": (_P, [_P]),
    "scrust_csr_free": (None, [_P]),
    "scrust_cuda_synchronize": (ctypes.c_int32, [_P, ctypes.POINTER(Status)]),
    "scrust_cuda_smooth_knn_distances_noalloc": (ctypes.c_int32, [_P, ctypes.c_uint64, ctypes.c_uint32, _P, _P,
                                                                   _P, ctypes.POINTER(Status)]),
    "scrust_cuda_set_timing": (None, [_P, ctypes.c_int32]),
    "scrust_cuda_phase_times": (ctypes.c_int32, [_P, ctypes.POINTER(ctypes.c_float), ctypes.c_int32]),
    "scrust_cuda_launch_count": (ctypes.c_uint64, [_P]),
    "scrust_cuda_selftest_bounded_wait": (ctypes.c_int32, [_P, ctypes.c_uint64, ctypes.POINTER(Status)]),
    "scrust_cuda_kernel_stats": (ctypes.c_int32, [_P, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64),
                                                   ctypes.c_int32]),
    "scrust_cuda_knn_batch": (ctypes.c_int32, [_P, _P, _P, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32,
                                                ctypes.POINTER(KnnOptions), _P, _P, ctypes.POINTER(Status)]),
    "scrust_cuda_knn_batch_device": (ctypes.c_int32, [_P, _P, _P, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32,
                                                       ctypes.POINTER(KnnOptions), _P, _P, ctypes.POINTER(Status)]),
    "scrust_cuda_batch_plan_create": (_P, [_P, _P, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32,
                                           ctypes.POINTER(KnnOptions), _P, _P, _P, ctypes.POINTER(Status)]),
    "scrust_cuda_batch_plan_launch": (ctypes.c_int32, [_P, ctypes.POINTER(Status)]),
    "scrust_cuda_batch_plan_choice": (ctypes.c_int32, [_P, ctypes.POINTER(ctypes.c_uint32),
                                                        ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_float)]),
    "scrust_cuda_batch_plan_destroy": (None, [_P]),
    "scrust_cuda_batch_plan_topk_width": (ctypes.c_int32, [_P]),
    "scrust_cuda_batch_plan_create_graphs": (_P, [_P, _P, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32,
                                                  ctypes.POINTER(KnnOptions), _P, _P, _P, ctypes.POINTER(Status)]),
    "scrust_cuda_batch_plan_graph": (ctypes.c_int32, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P),
                                                       ctypes.POINTER(_P)]),
    "scrust_cuda_neighbors_graph_batch": (ctypes.c_int32, [_P, _P, _P, ctypes.c_uint32, ctypes.c_uint64,
                                                            ctypes.c_uint32, ctypes.POINTER(KnnOptions), _P, _P,
                                                            ctypes.POINTER(_P), ctypes.POINTER(Status)]),
    "scrust_serve_create": (_P, [ctypes.c_int32, _P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                 ctypes.POINTER(KnnOptions), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                 ctypes.POINTER(Status)]),
    "scrust_serve_submit": (ctypes.c_uint64, [_P, _P, ctypes.c_uint64, ctypes.POINTER(Status)]),
    "scrust_serve_wait": (ctypes.c_int32, [_P, ctypes.c_uint64, _P, _P, ctypes.POINTER(_P),
                                           ctypes.POINTER(ctypes.c_double), ctypes.POINTER(Status)]),
    "scrust_serve_stats": (ctypes.c_int32, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.c_int32]),
    "scrust_serve_destroy": (None, [_P]),
    "scrust_cuda_knn_rows_device": (ctypes.c_int32, [_P, _P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                                      ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(KnnOptions),
                                                      _P, _P, ctypes.POINTER(Status)]),
    "scrust_cuda_version": (ctypes.c_char_p, []),
    "scrust_umap_params_default": (None, [ctypes.POINTER(UmapParams)]),
    "scrust_cuda_pca": (ctypes.c_int32, [_P, _P, _P, _P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                          ctypes.c_int32, ctypes.c_uint64, _P, _P, _P, _P, ctypes.POINTER(Status)]),
    "scrust_cuda_pca_device": (ctypes.c_int32, [_P, _P, _P, _P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                                 ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64, _P, _P, _P, _P,
                                                 ctypes.POINTER(Status)]),
    "scrust_cuda_leiden": (ctypes.c_int32, [_P, _P, _P, _P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double,
                                             ctypes.c_uint32, ctypes.c_uint64, _P, ctypes.POINTER(ctypes.c_double),
                                             ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(Status)]),
    "scrust_cuda_louvain": (ctypes.c_int32, [_P, _P, _P, _P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_double,
                                              ctypes.c_uint64, _P, ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(Status)]),
    "scrust_cuda_modularity": (ctypes.c_int32, [_P, _P, _P, _P, ctypes.c_uint64, ctypes.c_uint64, _P,
                                                 ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                                 ctypes.POINTER(Status)]),
    "scrust_cuda_umap": (ctypes.c_int32, [_P, _P, _P, _P, ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(UmapParams),
                                           _P, ctypes.POINTER(Status)]),
    "scrust_cuda_umap_device": (ctypes.c_int32, [_P, _P, _P, _P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                                  ctypes.POINTER(UmapParams), _P, ctypes.POINTER(Status)]),
}


def declared_symbols() -> list[str]:
    """Names of every function include/scrust_cuda.h declares."""
    import re

    header = pathlib.Path(__file__).resolve().parent.parent / "include" / "scrust_cuda.h"
    return re.findall(r"^SCRUST_API[^(]*?\b(scrust_\w+)\(", header.read_text(), flags=re.M)


def lib():
    """The loaded library (raises ImportError if it is not built)."""
    global _LIB
    with _LOCK:
        if _LIB is None:
            if not LIB_PATH.exists():
                raise ImportError(
                    f"{LIB_PATH} is not built; run `python -m mrustsc_gb300.build` (needs nvcc)"
                )
            handle = ctypes.CDLL(str(LIB_PATH))
            for name, (res, args) in _SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _LIB = handle
    return _LIB


def check(rc: int, status: Status) -> None:
    if rc == OK:
        return
    msg = status.message.decode(errors="replace") or f"status {rc}"
    if rc in (SHAPE, INVALID_PARAMETER):
        raise ScrustValueError(rc, msg)
    raise ScrustError(rc, msg)


def gpu_available() -> bool:
    return bool(lib().scrust_cuda_gpu_available())


def context(device: int = 0) -> int:
    """A process-wide context per device (the library serialises calls on it)."""
    with _LOCK:
        ctx = _CONTEXTS.get(device)
    if ctx:
        return ctx
    st = Status()
    handle = lib().scrust_cuda_context_create(device, ctypes.byref(st))
    if not handle:
        check(st.code or NO_GPU, st)
    with _LOCK:
        if device in _CONTEXTS:
            lib().scrust_cuda_context_destroy(handle)
        else:
            _CONTEXTS[device] = handle
        return _CONTEXTS[device]


def options(form: str | int = "auto", metric: str | int = "euclidean", mode: str | int = "exact",
            precision: str | int = "fp16", list_capacity: int = 0, segments: int = 0,
            ordering: str | int = "auto") -> KnnOptions:
    o = KnnOptions()
    lib().scrust_knn_options_default(ctypes.byref(o))

    def pick(table, value, what):
        if isinstance(value, str):
            if value not in table:
                raise ValueError(f"{what} must be one of {sorted(table)}, got {value!r}")
            return table[value]
        return int(value)

    o.form = pick(FORMS, form, "form")
    o.metric = pick(METRICS, metric, "metric")
    o.mode = pick(MODES, mode, "mode")
    o.precision = pick(PRECISIONS, precision, "precision")
    o.list_capacity = int(list_capacity)
    o.segments = int(segments)
    o.ordering = pick(ORDERINGS, ordering, "ordering")
    return o


def ptr(array: np.ndarray) -> int:
    return array.ctypes.data


def csr_host_arrays(handle) -> tuple[np.ndarray, np.ndarray, np.ndarray, int]:
    """Copies a host CSR handle into numpy arrays and frees the handle."""
    L = lib()
    try:
        n = int(L.scrust_csr_n_rows(handle))
        nnz = int(L.scrust_csr_nnz(handle))
        ncols = int(L.scrust_csr_n_cols(handle))

        def grab(p, count, ctype, dtype):
            if count == 0:
                return np.zeros(0, dtype=dtype)
            buf = (ctype * count).from_address(p)
            return np.frombuffer(buf, dtype=dtype, count=count).copy()

        indptr = grab(L.scrust_csr_indptr(handle), n + 1, ctypes.c_uint32, np.uint32)
        indices = grab(L.scrust_csr_indices(handle), nnz, ctypes.c_uint32, np.uint32)
        values = grab(L.scrust_csr_values(handle), nnz, ctypes.c_float, np.float32)
        return indptr, indices, values, ncols
    finally:
        L.scrust_csr_free(handle)
