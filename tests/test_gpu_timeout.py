"""Bounded device waits.  Every mbarrier wait of the sweep kernels gives up
after a wall-clock limit, sets the device error block's timeout flag and lets
the kernel return; the host reports SCRUST_TIMEOUT.  The self-test kernel
runs that wait on an mbarrier nothing arrives on (no copy and no MMA in
flight), so the path is exercised without hanging or faulting the GPU."""

from __future__ import annotations

import ctypes
import time

import numpy as np
import pytest

from mrustsc_gb300 import synthetic

pytestmark = pytest.mark.gpu


def test_a_wait_that_runs_out_is_a_timeout_status_and_the_context_stays_usable(built_library, oracle):
    from mrustsc_gb300 import _lib, _scrust

    L = _lib.lib()
    ctx = _lib.context(0)
    st = _lib.Status()
    t0 = time.perf_counter()
    rc = L.scrust_cuda_selftest_bounded_wait(ctx, 2_000_000, ctypes.byref(st))
    elapsed = time.perf_counter() - t0
    assert rc == _lib.TIMEOUT, (rc, st.message)
    assert b"bounded device wait ran out" in st.message
    assert elapsed < 5.0
    # The flag was cleared and the context still solves exactly.
    x = synthetic.mixture(3000, 30, clusters=6, dup_frac=0.01, seed=5)
    idx, _ = _scrust.knn(x, 10, "auto")
    oi, _, _ = oracle.knn_fp64(x, 10)
    np.testing.assert_array_equal(idx, oi)
    assert L.scrust_cuda_synchronize(ctx, ctypes.byref(st)) == _lib.OK


def test_the_self_test_takes_only_short_limits(built_library):
    from mrustsc_gb300 import _lib

    L = _lib.lib()
    st = _lib.Status()
    for bad in (0, 100_000_001):
        assert L.scrust_cuda_selftest_bounded_wait(_lib.context(0), bad, ctypes.byref(st)) == _lib.INVALID_PARAMETER
