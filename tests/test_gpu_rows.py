"""Row-range solves (one shard of a sharded graph build) on the GPU: the
shards' rows equal the single solve's rows bit for bit and the FP64 oracle."""

from __future__ import annotations

import numpy as np
import pytest

from mrustsc_gb300 import distributed, synthetic

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [1, 2, 3])
def test_shards_equal_the_whole_solve(built_library, oracle, world):
    from mrustsc_gb300 import _scrust

    x = synthetic.mixture(5000, 40, clusters=9, dup_frac=0.02, seed=11)
    k = 15
    whole_i, whole_d = _scrust.knn(x, k, "auto", form="tensor")
    parts = [distributed.knn_rows_gpu(x, k, *distributed.shard_rows(len(x), world, r)) for r in range(world)]
    idx = np.concatenate([p[0] for p in parts])
    dist = np.concatenate([p[1] for p in parts])
    np.testing.assert_array_equal(idx, whole_i)
    np.testing.assert_array_equal(dist, whole_d)
    oi, _, _ = oracle.knn_fp64(x, k)
    np.testing.assert_array_equal(idx, oi)


def test_row_range_arguments(built_library):
    import ctypes

    from mrustsc_gb300 import _lib

    L = _lib.lib()
    st = _lib.Status()
    ctx = _lib.context(0)
    rc = L.scrust_cuda_knn_rows_device(ctx, None, 100, 8, 5, 50, 40, None, None, None, ctypes.byref(st))
    assert rc == _lib.SHAPE
    rc = L.scrust_cuda_knn_rows_device(ctx, None, 100, 8, 100, 0, 10, None, None, None, ctypes.byref(st))
    assert rc == _lib.INVALID_PARAMETER
