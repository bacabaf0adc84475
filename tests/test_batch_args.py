"""Argument checks of the batched kNN entry points (no GPU needed)."""

from __future__ import annotations

import numpy as np
import pytest

from mrustsc_gb300 import _lib


@pytest.fixture(scope="module")
def scrust(built_library):
    from mrustsc_gb300 import _scrust

    return _scrust


def test_batch_rejects_bad_shapes(scrust):
    a = np.zeros((50, 8), np.float32)
    with pytest.raises(ValueError, match="every sample"):
        scrust.knn_batch([a, np.zeros((10, 8), np.float32)], 15, "auto")
    with pytest.raises(ValueError, match="same number of dimensions"):
        scrust.knn_batch([a, np.zeros((50, 9), np.float32)], 5, "auto")
    with pytest.raises(ValueError, match="61 dimensions"):
        scrust.knn_batch([np.zeros((50, 62), np.float32)], 5, "auto")
    with pytest.raises(ValueError, match="at least one sample"):
        scrust.knn_batch([], 5, "auto")
    with pytest.raises(ValueError):
        scrust.knn_batch([a], 0, "auto")


def test_batch_symbols_exported(built_library):
    L = _lib.lib()
    for name in ("scrust_cuda_knn_batch", "scrust_cuda_knn_batch_device", "scrust_cuda_batch_plan_create",
                 "scrust_cuda_batch_plan_launch", "scrust_cuda_batch_plan_choice", "scrust_cuda_batch_plan_destroy"):
        assert hasattr(L, name)
    assert L.scrust_cuda_batch_plan_choice(None, None, None, None) == 0
    L.scrust_cuda_batch_plan_destroy(None)
