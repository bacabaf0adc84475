"""The C ABI loads, exports every entry point include/scrust_cuda.h declares,
and rejects bad arguments the way the reference does -- before any device is
touched, so these run without a GPU."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest


@pytest.fixture(scope="module")
def L(built_library):
    from mrustsc_gb300 import _lib

    return _lib


def test_library_exports_every_declared_symbol(L):
    names = L.declared_symbols()
    assert len(names) >= 20
    handle = ctypes.CDLL(str(L.LIB_PATH))
    missing = [n for n in names if not hasattr(handle, n)]
    assert not missing, missing
    assert set(names) <= set(L._SIGNATURES)


def test_version_string(L):
    assert b"sm_103a" in L.lib().scrust_cuda_version()


def test_options_defaults(L):
    o = L.KnnOptions()
    L.lib().scrust_knn_options_default(ctypes.byref(o))
    assert o.struct_size == ctypes.sizeof(L.KnnOptions)
    assert (o.metric, o.mode, o.precision) == (0, 0, 0)


def _knn(L, n, d, k, ctx=None, opts=None):
    st = L.Status()
    x = np.zeros((max(n, 1), max(d, 1)), np.float32)
    idx = np.zeros(max(n * k, 1), np.uint32)
    dist = np.zeros(max(n * k, 1), np.float32)
    rc = L.lib().scrust_cuda_knn(ctx, L.ptr(x), n, d, k, ctypes.byref(opts) if opts else None, L.ptr(idx),
                                 L.ptr(dist), ctypes.byref(st))
    return rc, st.message.decode()


@pytest.mark.parametrize(("n", "d", "k", "code"), [
    (0, 4, 3, 1),      # neighbors.rs:42-47 Shape
    (5, 0, 3, 1),
    (6, 1, 0, 2),      # :48-50 InvalidParameter
    (6, 1, 6, 2),      # :51-57 k >= n
    (6, 1, 7, 2),
    (500, 2, 129, 2),  # above max_supported_k
])
def test_knn_rejects_degenerate_arguments(L, n, d, k, code):
    rc, msg = _knn(L, n, d, k)
    assert rc == code, msg
    assert msg


def test_valid_arguments_without_a_context_report_no_gpu(L):
    rc, msg = _knn(L, 10, 2, 3)
    assert rc == L.NO_GPU
    assert "GPU" in msg


def test_bad_options_are_invalid_parameters(L):
    o = L.options(metric="cosine", mode="reference_snap")
    rc, msg = _knn(L, 10, 2, 3, opts=o)
    assert rc == L.INVALID_PARAMETER and "cosine" in msg
    o = L.options()
    o.form = 9
    rc, _ = _knn(L, 10, 2, 3, opts=o)
    assert rc == L.INVALID_PARAMETER


def test_connectivities_validation_matches_the_reference(L):
    st = L.Status()
    out = ctypes.c_void_p()
    idx = np.array([[1], [9]], np.uint32)
    dist = np.ones((2, 1), np.float32)
    rc = L.lib().scrust_cuda_connectivities(None, L.ptr(idx), L.ptr(dist), 2, 1, ctypes.byref(out), ctypes.byref(st))
    assert rc == L.SHAPE and "out-of-range" in st.message.decode()
    rc = L.lib().scrust_cuda_connectivities(None, L.ptr(idx), L.ptr(dist), 0, 1, ctypes.byref(out), ctypes.byref(st))
    assert rc == L.SHAPE


def test_null_context_accessors_are_safe(L):
    lib = L.lib()
    assert lib.scrust_cuda_max_supported_k(None) == 0
    assert lib.scrust_cuda_context_stream(None) is None
    assert lib.scrust_csr_nnz(None) == 0
    lib.scrust_csr_free(None)
    lib.scrust_cuda_context_destroy(None)


def test_python_layer_maps_errors_like_the_reference(L):
    from mrustsc_gb300 import _scrust

    with pytest.raises(ValueError, match="2-D numpy array of float32"):
        _scrust.knn(np.zeros((4, 2), np.float64), 1, "auto")
    with pytest.raises(ValueError, match="2-D numpy array of float32"):
        _scrust.knn(np.zeros(4, np.float32), 1, "auto")
    with pytest.raises(ValueError):
        _scrust.knn(np.zeros((6, 1), np.float32), 6, "auto")
    with pytest.raises(ValueError, match="cpu"):
        _scrust.knn(np.zeros((6, 1), np.float32), 2, "cpu")
    with pytest.raises(ValueError, match="uint32"):
        _scrust.connectivities(np.zeros((2, 1), np.int64), np.zeros((2, 1), np.float32))
    with pytest.raises(ValueError):
        _scrust.connectivities(np.zeros((2, 1), np.uint32), np.zeros((2, 2), np.float32))


def test_bounded_wait_self_test_needs_a_context(L):
    st = L.Status()
    assert L.lib().scrust_cuda_selftest_bounded_wait(None, 1_000_000, ctypes.byref(st)) == L.NO_GPU
