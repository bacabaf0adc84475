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
