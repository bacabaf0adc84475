"""The allocation-free smooth_knn entry point (collected last on purpose).

scrust_cuda_smooth_knn_distances_noalloc serves callers that cannot let a
library call cudaMalloc -- a process whose pool allocator owns all device
memory, or a service that fixes its HBM budget at start-up.  They pass
device buffers they own; the entry point's scratch is a fixed array compiled
into the library.  Its results must match the regular entry point's and the
oracle's within the tolerances the other connectivities tests use (rho exact,
sigma 1e-5 relative against the regular entry point and 5e-5 against the
host restatement), on two calls in a row (the scratch keeps the previous
call's contents), up to the largest accepted size; a call must leave the
device's free memory unchanged; inputs beyond the array's limit and buffers
that are not device memory of one GPU must be refused.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIGMA_RTOL = 1e-5
# Against the host restatement: CUDA's expf and the host's differ by an ulp on
# some terms, which can move the bisection's stop (|cardinality - target| <
# 1e-5) by one step; sigma then moves by up to about 2e-5 relative.
SIGMA_ORACLE_RTOL = 5e-5
MAX_ENTRIES = 16_777_216  # n * k the scratch array serves


def _noalloc(L, _lib, torch, d_dist, n, k, sig, rho):
    st = _lib.Status()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.scrust_cuda_smooth_knn_distances_noalloc(d_dist.data_ptr(), n, k, sig.data_ptr(), rho.data_ptr(),
                                                    stream, ctypes.byref(st))
    return rc, st


def _run_twice(L, _lib, torch, dist, check):
    n, k = dist.shape
    d_dist = torch.from_numpy(dist).cuda()
    sig = torch.empty(n, dtype=torch.float32, device="cuda")
    rho = torch.empty(n, dtype=torch.float32, device="cuda")
    for _call in range(2):
        sig.fill_(-1.0)
        rho.fill_(-1.0)
        rc, st = _noalloc(L, _lib, torch, d_dist, n, k, sig, rho)
        _lib.check(rc, st)
        torch.cuda.synchronize()
        check(sig.cpu().numpy(), rho.cpu().numpy())


@pytest.mark.parametrize("duplicates", [False, True])
def test_noalloc_matches_the_allocating_entry_point_and_the_oracle_twice(built_library, oracle, duplicates):
    import torch

    from mrustsc_gb300 import _lib, _scrust, synthetic

    L = _lib.lib()
    assert _scrust.gpu_available(), "this test needs an sm_103a GPU"
    x = synthetic.plain_small(seed=5)
    if duplicates:
        x[:40] = x[0]  # rows whose neighbours are all at distance 0 use the global mean
    k = 15
    _, dist = _scrust.knn(x, k, "auto")
    sig_ref, rho_ref = _scrust.smooth_knn_distances(dist)
    sig_cpu, rho_cpu = oracle.smooth_knn(dist)

    def check(sig, rho):
        np.testing.assert_array_equal(rho, rho_ref)
        np.testing.assert_allclose(sig, sig_ref, rtol=SIGMA_RTOL, atol=0)
        np.testing.assert_array_equal(rho, rho_cpu)
        np.testing.assert_allclose(sig, sig_cpu, rtol=SIGMA_ORACLE_RTOL, atol=0)

    _run_twice(L, _lib, torch, dist, check)


def test_noalloc_at_the_largest_accepted_size(built_library):
    """n * k = 16,777,216 exactly (1,048,576 rows of 16), with rows of zeros."""
    import torch

    from mrustsc_gb300 import _lib, _scrust

    L = _lib.lib()
    n, k = MAX_ENTRIES // 16, 16
    rng = np.random.default_rng(7)
    dist = np.sort(rng.gamma(2.0, 1.0, size=(n, k)).astype(np.float32), axis=1)
    dist[:: 997] = 0.0
    dist[5::1013, :3] = 0.0
    sig_ref, rho_ref = _scrust.smooth_knn_distances(dist)

    def check(sig, rho):
        np.testing.assert_array_equal(rho, rho_ref)
        np.testing.assert_allclose(sig, sig_ref, rtol=SIGMA_RTOL, atol=0)

    _run_twice(L, _lib, torch, dist, check)


def test_noalloc_leaves_device_memory_untouched(built_library):
    import torch

    from mrustsc_gb300 import _lib

    L = _lib.lib()
    n, k = 50_000, 15
    dist = np.sort(np.random.default_rng(3).random((n, k), dtype=np.float32), axis=1)
    d_dist = torch.from_numpy(dist).cuda()
    sig = torch.empty(n, dtype=torch.float32, device="cuda")
    rho = torch.empty(n, dtype=torch.float32, device="cuda")
    _lib.check(*_noalloc(L, _lib, torch, d_dist, n, k, sig, rho))  # first call: address look-up
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        _lib.check(*_noalloc(L, _lib, torch, d_dist, n, k, sig, rho))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_noalloc_refuses_inputs_beyond_its_scratch(built_library):
    import torch

    from mrustsc_gb300 import _lib

    L = _lib.lib()
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    st = _lib.Status()
    rc = L.scrust_cuda_smooth_knn_distances_noalloc(buf.data_ptr(), 1 << 22, 5, buf.data_ptr(), buf.data_ptr(),
                                                    None, ctypes.byref(st))
    assert rc == _lib.INVALID_PARAMETER
    assert "16777216" in st.message.decode()


def test_noalloc_refuses_buffers_that_are_not_device_memory(built_library):
    import torch

    from mrustsc_gb300 import _lib

    L = _lib.lib()
    host = np.zeros((4, 2), np.float32)
    dev = torch.zeros(8, dtype=torch.float32, device="cuda")
    st = _lib.Status()
    rc = L.scrust_cuda_smooth_knn_distances_noalloc(_lib.ptr(host), 4, 2, dev.data_ptr(), dev.data_ptr(), None,
                                                    ctypes.byref(st))
    assert rc == _lib.INVALID_PARAMETER
    assert "device memory" in st.message.decode()
