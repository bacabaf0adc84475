"""The sharded graph build's host logic on two gloo ranks (CPU).

Each rank solves its rows with the FP64 oracle; the gathered graph and its
connectivities must equal the single-process oracle's bit for bit.
"""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from mrustsc_gb300 import distributed, synthetic


def test_shard_rows_cover_every_row_once():
    for n in (1, 2, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            spans = [distributed.shard_rows(n, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        distributed.shard_rows(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist

    from oracle import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        x = synthetic.mixture(600, 12, clusters=4, dup_frac=0.05, seed=7)

        def rows(x_, k_, r0, r1):
            idx, _, dist_f32 = oracle.knn_fp64(x_, k_, np.arange(r0, r1))
            return idx.astype(np.uint32), dist_f32

        def conn(idx, dist_):
            indptr, cols, vals, _ = oracle.connectivities(idx, dist_)
            return indptr, cols, vals

        res = distributed.neighbors_sharded(x, 9, rank, world, knn_rows=rows, connectivities=conn)
        if rank == 0:
            np.savez(out, idx=res[0], dist=res[1], indptr=res[2][0], cols=res[2][1], vals=res[2][2])
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_equal_one_process(tmp_path, oracle):
    import torch.multiprocessing as mp

    out = str(tmp_path / "sharded.npz")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    got = np.load(out)
    x = synthetic.mixture(600, 12, clusters=4, dup_frac=0.05, seed=7)
    idx, _, dist = oracle.knn_fp64(x, 9)
    np.testing.assert_array_equal(got["idx"], idx.astype(np.uint32))
    np.testing.assert_array_equal(got["dist"], dist)
    indptr, cols, vals, _ = oracle.connectivities(idx.astype(np.uint32), dist)
    np.testing.assert_array_equal(got["indptr"], indptr)
    np.testing.assert_array_equal(got["cols"], cols)
    np.testing.assert_array_equal(got["vals"], vals)


def test_default_row_solver_runs_on_the_ranks_current_device(monkeypatch):
    """With no solver passed, each rank solves its rows on its own GPU (the
    current CUDA device of its process), never on device 0 by default."""
    import torch

    seen = {}

    def fake_upload(x, device):
        seen["upload"] = device
        return torch.from_numpy(np.ascontiguousarray(x))

    def fake_rows_device(xd, k, r0, r1, precision="fp16"):
        seen["rows"] = (r0, r1)
        return torch.zeros((r1 - r0, k), dtype=torch.int32), torch.zeros((r1 - r0, k), dtype=torch.float32)

    monkeypatch.setattr(torch.cuda, "current_device", lambda: 3)
    monkeypatch.setattr(distributed, "_upload", fake_upload)
    monkeypatch.setattr(distributed, "knn_rows_device", fake_rows_device)
    monkeypatch.setattr(distributed, "gather_rows", lambda block, n, world, group=None: block)
    monkeypatch.setattr(distributed, "_collective_device", lambda group: torch.device("cpu"))
    x = np.zeros((10, 4), np.float32)
    distributed.neighbors_sharded(x, 2, rank=1, world=2, connectivities=lambda i, d: None)
    assert seen == {"upload": 3, "rows": (5, 10)}
    seen.clear()
    distributed.knn_rows_gpu(x, 2, 0, 5)
    assert seen == {"upload": 3, "rows": (0, 5)}
