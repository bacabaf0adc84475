"""The allocation-free smooth_knn entry point (collected last on purpose).

scrust_cuda_smooth_knn_distances_noalloc serves callers that cannot let a
library call cudaMalloc -- a process whose pool allocator owns all device
memory, or a service that fixes its HBM budget at start-up.  They pass
device buffers they own; the entry point's scratch is a fixed array compiled
into the library.  Its results must match the regular entry point's within
the tolerance the other connectivities tests use (rho exact, sigma 1e-5
relative), on two calls in a row (the scratch keeps the previous call's
contents), and inputs beyond the array's limit must be refused.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIGMA_RTOL = 1e-5


def _noalloc(L, _lib, torch, d_dist, n, k, sig, rho):
    st = _lib.Status()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.scrust_cuda_smooth_knn_distances_noalloc(d_dist.data_ptr(), n, k, sig.data_ptr(), rho.data_ptr(),
                                                    stream, ctypes.byref(st))
    return rc, st


@pytest.mark.parametrize("duplicates", [False, True])
def test_noalloc_matches_the_allocating_entry_point_twice(built_library, duplicates):
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
    n = dist.shape[0]
    d_dist = torch.from_numpy(dist).cuda()
    sig = torch.empty(n, dtype=torch.float32, device="cuda")
    rho = torch.empty(n, dtype=torch.float32, device="cuda")
    for _call in range(2):
        sig.fill_(-1.0)
        rho.fill_(-1.0)
        rc, st = _noalloc(L, _lib, torch, d_dist, n, k, sig, rho)
        _lib.check(rc, st)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(rho.cpu().numpy(), rho_ref)
        np.testing.assert_allclose(sig.cpu().numpy(), sig_ref, rtol=SIGMA_RTOL, atol=0)


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
