"""Batched kNN (many independent samples in one tensor sweep) on the GPU.

Every sample's neighbour lists and distances must be the same bits as a
solve of that sample alone, and equal to the FP64 oracle.  The batching
form has no reference counterpart; parity is against FP64 and the
single-sample path.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from mrustsc_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scrust(built_library):
    from mrustsc_gb300 import _scrust

    assert _scrust.gpu_available(), "these tests need an sm_103a GPU"
    return _scrust


def ragged_samples(sizes, d=50, seed=0):
    return [synthetic.mixture(n, d, clusters=4 + s % 7, dup_frac=0.01, seed=seed * 100 + s)
            for s, n in enumerate(sizes)]


@pytest.mark.parametrize("k", [15, 30])
def test_batch_equals_single_sample_solves_and_fp64(scrust, oracle, k):
    samples = ragged_samples([300, 1000, 257, 256, 3000, 40, 511, 2049], seed=k)
    out = scrust.knn_batch(samples, k, "auto")
    for x, (idx, dist) in zip(samples, out):
        si, sd = scrust.knn(x, k, "auto", form="tensor")
        np.testing.assert_array_equal(idx, si)
        np.testing.assert_array_equal(dist, sd)
        pi, pd = scrust.knn(x, k, "auto", form="plain")
        np.testing.assert_array_equal(idx, pi)
        np.testing.assert_array_equal(dist, pd)
        oi, od64, _ = oracle.knn_fp64(x, k)
        np.testing.assert_array_equal(idx, oi)


def test_batch_cosine_and_bf16(scrust, oracle):
    samples = ragged_samples([700, 129, 1500], seed=3)
    for kwargs in ({"metric": "cosine"}, {"precision": "bf16"}):
        out = scrust.knn_batch(samples, 12, "auto", **kwargs)
        for x, (idx, dist) in zip(samples, out):
            metric = kwargs.get("metric", "euclidean")
            oi, _, od = oracle.knn_fp64(x, 12, metric=metric)
            np.testing.assert_array_equal(idx, oi)
            si, sd = scrust.knn(x, 12, "auto", form="plain", metric=metric)
            np.testing.assert_array_equal(dist, sd)


def test_batch_of_one_and_duplicates(scrust, oracle):
    x = synthetic.mixture(900, 20, clusters=3, dup_frac=0.2, seed=9)
    (idx, dist), = scrust.knn_batch([x], 14, "auto")
    si, sd = scrust.knn(x, 14, "auto", form="plain")
    np.testing.assert_array_equal(idx, si)
    np.testing.assert_array_equal(dist, sd)


def test_plan_graph_launch_matches_direct_batch(scrust):
    torch = pytest.importorskip("torch")
    samples = ragged_samples([600, 2500, 300, 1200], seed=5)
    k = 15
    direct = scrust.knn_batch(samples, k, "auto")
    x = np.concatenate(samples)
    offsets = np.zeros(len(samples) + 1, dtype=np.uint64)
    offsets[1:] = np.cumsum([len(s) for s in samples])
    L = _lib.lib()
    ctx = _lib.context(0)
    xd = torch.from_numpy(x).cuda()
    idx = torch.empty((len(x), k), dtype=torch.int32, device="cuda")
    dst = torch.empty((len(x), k), dtype=torch.float32, device="cuda")
    st = _lib.Status()
    opts = _lib.options(form="tensor")
    plan = L.scrust_cuda_batch_plan_create(ctx, _lib.ptr(offsets), len(samples), x.shape[1], k, ctypes.byref(opts),
                                           xd.data_ptr(), idx.data_ptr(), dst.data_ptr(), ctypes.byref(st))
    assert plan, st.message.decode()
    try:
        cap, prec, ms = ctypes.c_uint32(), ctypes.c_int32(), ctypes.c_float()
        assert L.scrust_cuda_batch_plan_choice(plan, ctypes.byref(cap), ctypes.byref(prec), ctypes.byref(ms)) == 1
        assert cap.value in (64, 128, 256) and prec.value in (0, 1) and ms.value > 0
        for _ in range(2):
            idx.zero_()
            _lib.check(L.scrust_cuda_batch_plan_launch(plan, ctypes.byref(st)), st)
            _lib.check(L.scrust_cuda_synchronize(ctx, ctypes.byref(st)), st)
            gi = idx.cpu().numpy().view(np.uint32)
            gd = dst.cpu().numpy()
            for s, (di, dd) in enumerate(direct):
                a, b = int(offsets[s]), int(offsets[s + 1])
                np.testing.assert_array_equal(gi[a:b], di)
                np.testing.assert_array_equal(gd[a:b], dd)
    finally:
        L.scrust_cuda_batch_plan_destroy(plan)


@pytest.mark.parametrize("k", [15, 30])
def test_batch_graphs_equal_single_sample_graphs(scrust, oracle, k):
    """Every sample's connectivities from the batch pass equal the restated
    connectivities of that sample's own kNN graph (CSR structure bit-exact,
    values within 1e-5), and the kNN rows equal the single-sample solve."""
    samples = ragged_samples([300, 1000, 257, 3000, 40, 511, 2049], seed=k + 1)
    samples[3][100:260] = samples[3][100]  # hub rows inside one sample
    out = scrust.neighbors_graph_batch(samples, k, "auto")
    for x, (idx, dist, csr) in zip(samples, out):
        si, sd = scrust.knn(x, k, "auto", form="tensor")
        np.testing.assert_array_equal(idx, si)
        np.testing.assert_array_equal(dist, sd)
        ref = oracle.connectivities(idx, dist)
        np.testing.assert_array_equal(csr[0], ref[0])
        np.testing.assert_array_equal(csr[1], ref[1])
        np.testing.assert_allclose(csr[2], ref[2], rtol=0, atol=1e-5)
        assert csr[3] == len(x)


def test_graph_plan_builds_every_sample_in_one_launch(scrust, oracle):
    import torch

    L = _lib.lib()
    ctx = _lib.context(0)
    samples = ragged_samples([700, 2500, 260, 1200], seed=9)
    k = 15
    x = np.concatenate(samples)
    offsets = np.zeros(len(samples) + 1, np.uint64)
    offsets[1:] = np.cumsum([len(s) for s in samples])
    n = int(offsets[-1])
    xd = torch.from_numpy(x).cuda()
    idx = torch.empty((n, k), dtype=torch.int32, device="cuda")
    dst = torch.empty((n, k), dtype=torch.float32, device="cuda")
    st = _lib.Status()
    opts = _lib.options(form="tensor")
    plan = L.scrust_cuda_batch_plan_create_graphs(ctx, _lib.ptr(offsets), len(samples), 50, k, ctypes.byref(opts),
                                                  xd.data_ptr(), idx.data_ptr(), dst.data_ptr(), ctypes.byref(st))
    assert plan, st.message.decode()
    try:
        assert L.scrust_cuda_batch_plan_topk_width(plan) in (0, 16, 32)
        idx.fill_(0)
        _lib.check(L.scrust_cuda_batch_plan_launch(plan, ctypes.byref(st)), st)
        _lib.check(L.scrust_cuda_synchronize(ctx, ctypes.byref(st)), st)
        ip, ix, vl = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        assert L.scrust_cuda_batch_plan_graph(plan, ctypes.byref(ip), ctypes.byref(ix), ctypes.byref(vl)) == 1

        class DeviceView:  # the plan's device array, seen by torch without a copy
            def __init__(self, ptr, count, typestr):
                self.__cuda_array_interface__ = {"shape": (count,), "typestr": typestr, "data": (ptr, False),
                                                 "version": 2}

        def grab(ptr, count, typestr):
            return torch.as_tensor(DeviceView(ptr.value, count, typestr), device="cuda").cpu().numpy()

        indptr = grab(ip, n + 1, "<u4")
        nnz = int(indptr[-1])
        cols = grab(ix, nnz, "<u4")
        vals = grab(vl, nnz, "<f4")
        gi = idx.cpu().numpy().view(np.uint32)
        gd = dst.cpu().numpy()
        from mrustsc_gb300._scrust import split_batch_graph

        for xs, (si, sd, csr) in zip(samples, split_batch_graph(offsets, gi, gd, indptr, cols, vals)):
            np.testing.assert_array_equal(si, oracle.knn_fp64(xs, k)[0])
            ref = oracle.connectivities(si, sd)
            np.testing.assert_array_equal(csr[0], ref[0])
            np.testing.assert_array_equal(csr[1], ref[1])
            np.testing.assert_allclose(csr[2], ref[2], rtol=0, atol=1e-5)
    finally:
        L.scrust_cuda_batch_plan_destroy(plan)
