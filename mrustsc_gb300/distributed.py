"""A graph build sharded over several GPUs, one process per GPU.

kNN shards by query rows with no exchange: every rank holds the embedding
(200 MB at 1M x 50) and solves its block of rows against all of them
(`scrust_cuda_knn_rows_device`).  The connectivities need every row's
neighbours, so the rows' (ids, distances) are gathered, one n x k block of
12 bytes per entry, and the fuzzy union runs on one GPU; this keeps the
result bit-identical to a single-GPU build.

The gather is one `torch.distributed.all_gather` per array on tensors that
stay where the collective runs: device memory under NCCL (no host round
trip), host memory under gloo.  The row solver and the connectivity step are
passed in, so the same host logic runs with the GPU library or, in tests,
with any other row solver on CPU ranks.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def shard_rows(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous, balanced rows [r0, r1) of rank `rank` out of `world`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank must be in [0, {world}), got {rank}")
    base, extra = divmod(n, world)
    r0 = rank * base + min(rank, extra)
    return r0, r0 + base + (1 if rank < extra else 0)


def gather_rows(block, n: int, world: int, group=None):
    """All ranks' row blocks (each rank's from shard_rows), in row order.

    `block` is a torch tensor on the collective's device (CUDA for NCCL, CPU
    for gloo) of int32 or float32; the result is an (n, width) tensor on the
    same device.  Blocks differ in length by at most one row, so each is
    padded to the longest before the all_gather.
    """
    import torch
    import torch.distributed as dist

    per = -(-n // world)
    width = block.shape[1]
    pad = block.new_zeros((per, width))
    pad[: block.shape[0]] = block
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    pieces = []
    for r, p in enumerate(parts):
        a, b = shard_rows(n, world, r)
        pieces.append(p[: b - a])
    return torch.cat(pieces, dim=0)


def knn_rows_device(xd, k: int, r0: int, r1: int, precision: str = "fp16"):
    """Rows [r0, r1) of the exact kNN graph of the device-resident embedding
    `xd` (an (n, d) float32 CUDA tensor), on xd's GPU: (ids int32, distances
    float32) CUDA tensors of (r1 - r0, k), ready once the call returns."""
    import torch

    n, d = xd.shape
    device = xd.device.index if xd.device.index is not None else torch.cuda.current_device()
    L = _lib.lib()
    ctx = _lib.context(device)
    idx = torch.empty((r1 - r0, k), dtype=torch.int32, device=xd.device)
    dst = torch.empty((r1 - r0, k), dtype=torch.float32, device=xd.device)
    st = _lib.Status()
    opts = _lib.options(form="tensor", precision=precision)
    _lib.check(L.scrust_cuda_knn_rows_device(ctx, xd.data_ptr(), n, d, k, r0, r1, ctypes.byref(opts),
                                             idx.data_ptr(), dst.data_ptr(), ctypes.byref(st)), st)
    _lib.check(L.scrust_cuda_synchronize(ctx, ctypes.byref(st)), st)
    return idx, dst


def _upload(x, device: int):
    """The embedding as a float32 tensor on CUDA device `device`."""
    import torch

    if isinstance(x, torch.Tensor):
        return x.to(f"cuda:{device}")
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to(f"cuda:{device}")


def knn_rows_gpu(x: np.ndarray, k: int, r0: int, r1: int, device: int | None = None, precision: str = "fp16"):
    """Rows [r0, r1) of the exact kNN graph of the host array x on GPU
    `device` (default: this process's current CUDA device), as numpy."""
    import torch

    if device is None:
        device = torch.cuda.current_device()
    idx, dst = knn_rows_device(_upload(x, device), k, r0, r1, precision)
    return idx.cpu().numpy().view(np.uint32), dst.cpu().numpy()


def _collective_device(group):
    import torch
    import torch.distributed as dist

    if dist.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def neighbors_sharded(x, k: int, rank: int, world: int, group=None, knn_rows=None, connectivities=None,
                      root: int = 0):
    """Sharded kNN + gathered connectivities.

    `x` is the (n, d) embedding, a numpy array or a CUDA tensor already on
    this rank's GPU.  `knn_rows(x, k, r0, r1)` returns this rank's rows as
    numpy arrays or tensors; by default the library solves them on the
    rank's current CUDA device.  `connectivities(idx, dist)` takes the
    gathered (n, k) uint32 ids and float32 distances as numpy arrays; by
    default the library builds them on the root's GPU.  Returns (indices,
    distances, connectivities) on `root` -- numpy arrays and the reference's
    CSR tuple -- and (None, None, None) elsewhere.
    """
    import torch

    n = x.shape[0]
    r0, r1 = shard_rows(n, world, rank)
    if knn_rows is None:
        # This rank's GPU: one process per GPU, each with its device current.
        idx, dist = knn_rows_device(_upload(x, torch.cuda.current_device()), k, r0, r1)
    else:
        idx, dist = knn_rows(x, k, r0, r1)
    dev = _collective_device(group)

    def as_tensor(a, dtype):
        if isinstance(a, torch.Tensor):
            return a.to(dev)
        a = np.ascontiguousarray(a)
        return torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a.astype(dtype, copy=False)).to(dev)

    all_idx = gather_rows(as_tensor(idx, np.int32), n, world, group)
    all_dist = gather_rows(as_tensor(dist, np.float32), n, world, group)
    if rank != root:
        return None, None, None
    idx_np = all_idx.cpu().numpy().view(np.uint32)
    dist_np = all_dist.cpu().numpy()
    if connectivities is None:
        from . import _scrust

        connectivities = _scrust.connectivities
    return idx_np, dist_np, connectivities(idx_np, dist_np)


def neighbors_sharded_device(xd, k: int, rank: int, world: int, group=None, root: int = 0):
    """The device-resident form for one process per GPU under NCCL: the rows
    are solved on this rank's GPU, gathered into device tensors, and the root
    builds the connectivities there.  Returns (ids, distances, csr handle) on
    the root -- CUDA tensors of (n, k) and a device CSR (free it with
    scrust_csr_free) -- and (None, None, None) elsewhere."""
    import torch

    n = xd.shape[0]
    r0, r1 = shard_rows(n, world, rank)
    idx, dist = knn_rows_device(xd, k, r0, r1)
    all_idx = gather_rows(idx, n, world, group)
    all_dist = gather_rows(dist, n, world, group)
    if rank != root:
        return None, None, None
    torch.cuda.current_stream().synchronize()
    L = _lib.lib()
    ctx = _lib.context(xd.device.index if xd.device.index is not None else torch.cuda.current_device())
    st = _lib.Status()
    csr = ctypes.c_void_p()
    _lib.check(L.scrust_cuda_connectivities_device(ctx, all_idx.data_ptr(), all_dist.data_ptr(), n, k,
                                                   ctypes.byref(csr), ctypes.byref(st)), st)
    return all_idx, all_dist, csr
