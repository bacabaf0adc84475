"""A graph build sharded over several GPUs, one process per GPU.

kNN shards by query rows with no exchange: every rank holds the embedding
(200 MB at 1M x 50) and solves its block of rows against all of them
(`scrust_cuda_knn_rows_device`).  The connectivities need every row's
neighbours, so the rows' (ids, distances) are gathered, one n x k block of
12 bytes per entry, and the fuzzy union runs on one GPU; this keeps the
result bit-identical to a single-GPU build.  The collective is
`torch.distributed.all_gather` (NCCL between GPUs, gloo between CPU ranks);
the kNN and connectivity steps are passed in, so the same host logic runs
with the GPU library or, in tests, with any other row solver.
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


def gather_rows(block: np.ndarray, n: int, world: int, group=None) -> np.ndarray:
    """All ranks' row blocks (each rank's from shard_rows) in row order."""
    import torch
    import torch.distributed as dist

    per = -(-n // world)
    width = block.shape[1]
    pad = np.zeros((per, width), dtype=block.dtype)
    pad[: len(block)] = block
    backend = dist.get_backend(group)
    device = f"cuda:{torch.cuda.current_device()}" if backend == "nccl" else "cpu"
    t = torch.from_numpy(pad.view(np.int32) if block.dtype == np.uint32 else pad).to(device)
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    out = np.empty((n, width), dtype=block.dtype)
    for r, p in enumerate(parts):
        a, b = shard_rows(n, world, r)
        arr = p.cpu().numpy()
        out[a:b] = (arr.view(np.uint32) if block.dtype == np.uint32 else arr)[: b - a]
    return out


def knn_rows_gpu(x: np.ndarray, k: int, r0: int, r1: int, device: int = 0, precision: str = "fp16"):
    """Rows [r0, r1) of the exact kNN graph of x on this process's GPU."""
    import torch

    n, d = x.shape
    L = _lib.lib()
    ctx = _lib.context(device)
    xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to(f"cuda:{device}")
    idx = torch.empty((r1 - r0, k), dtype=torch.int32, device=xd.device)
    dst = torch.empty((r1 - r0, k), dtype=torch.float32, device=xd.device)
    st = _lib.Status()
    opts = _lib.options(form="tensor", precision=precision)
    _lib.check(L.scrust_cuda_knn_rows_device(ctx, xd.data_ptr(), n, d, k, r0, r1, ctypes.byref(opts),
                                             idx.data_ptr(), dst.data_ptr(), ctypes.byref(st)), st)
    _lib.check(L.scrust_cuda_synchronize(ctx, ctypes.byref(st)), st)
    return idx.cpu().numpy().view(np.uint32), dst.cpu().numpy()


def neighbors_sharded(x: np.ndarray, k: int, rank: int, world: int, group=None, knn_rows=None,
                      connectivities=None, root: int = 0):
    """Sharded kNN + gathered connectivities.

    Returns (indices, distances, connectivities) on `root` and (None, None,
    None) elsewhere; `knn_rows(x, k, r0, r1)` and `connectivities(idx, dist)`
    default to this library on the rank's GPU.
    """
    if knn_rows is None:
        knn_rows = knn_rows_gpu
    if connectivities is None:
        from . import _scrust

        connectivities = _scrust.connectivities
    n = x.shape[0]
    r0, r1 = shard_rows(n, world, rank)
    idx, dist = knn_rows(x, k, r0, r1)
    all_idx = gather_rows(np.ascontiguousarray(idx, dtype=np.uint32), n, world, group)
    all_dist = gather_rows(np.ascontiguousarray(dist, dtype=np.float32), n, world, group)
    if rank != root:
        return None, None, None
    return all_idx, all_dist, connectivities(all_idx, all_dist)
