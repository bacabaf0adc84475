"""The query service over a resident atlas (C ABI `scrust_serve_*`), and
its benchmark: a seeded Poisson stream of requests answered with continuous
batching, reporting p50/p99 latency and cells/s."""

from __future__ import annotations

import ctypes
import json
import threading
import time

import numpy as np

from . import _lib


class Server:
    """k nearest atlas cells plus directed connectivity rows for each request."""

    def __init__(self, atlas, k: int, device: int = 0, *, budget_bytes: int = 0, max_batch_cells: int = 0,
                 slots: int = 0, precision: str = "fp16"):
        self.atlas = np.ascontiguousarray(atlas, dtype=np.float32)
        self.m, self.d = self.atlas.shape
        self.k = int(k)
        L = _lib.lib()
        st = _lib.Status()
        opts = _lib.options(form="tensor", precision=precision)
        self._h = L.scrust_serve_create(device, _lib.ptr(self.atlas), self.m, self.d, self.k, ctypes.byref(opts),
                                        budget_bytes, max_batch_cells, slots, ctypes.byref(st))
        if not self._h:
            _lib.check(st.code or _lib.KERNEL, st)

    def submit(self, queries) -> int:
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if q.ndim != 2 or q.shape[1] != self.d:
            raise _lib.ScrustValueError(_lib.SHAPE, f"expected queries shaped (q, {self.d}), got {q.shape}")
        st = _lib.Status()
        t = _lib.lib().scrust_serve_submit(self._h, _lib.ptr(q), q.shape[0], ctypes.byref(st))
        if not t:
            _lib.check(st.code or _lib.KERNEL, st)
        return int(t), q.shape[0]

    def wait(self, ticket):
        t, q = ticket
        idx = np.empty((q, self.k), np.uint32)
        dist = np.empty((q, self.k), np.float32)
        csr = ctypes.c_void_p()
        lat = ctypes.c_double()
        st = _lib.Status()
        rc = _lib.lib().scrust_serve_wait(self._h, t, _lib.ptr(idx), _lib.ptr(dist), ctypes.byref(csr),
                                          ctypes.byref(lat), ctypes.byref(st))
        _lib.check(rc, st)
        indptr, indices, values, _ = _lib.csr_host_arrays(csr)  # frees the handle
        return idx, dist, (indptr, indices, values), lat.value

    def query(self, queries):
        return self.wait(self.submit(queries))

    def stats(self) -> dict:
        out = (ctypes.c_uint64 * 7)()
        _lib.lib().scrust_serve_stats(self._h, out, 7)
        keys = ["batches", "requests", "max_batches_in_flight", "cells", "max_batch_cells", "bytes_per_cell", "slots"]
        return dict(zip(keys, (int(v) for v in out)))

    def close(self):
        if self._h:
            _lib.lib().scrust_serve_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _replay(server: Server, times, queries):
    """Submits each request at its arrival time from one thread and waits for
    them from another; returns per-request latencies (ms) and the wall time."""
    tickets = [None] * len(times)
    lat = [0.0] * len(times)
    ready = [threading.Event() for _ in times]

    def waiter():
        for i in range(len(times)):
            ready[i].wait()
            lat[i] = server.wait(tickets[i])[3]

    th = threading.Thread(target=waiter)
    th.start()
    t0 = time.perf_counter()
    for i, (t, q) in enumerate(zip(times, queries)):
        now = time.perf_counter() - t0
        if t > now:
            time.sleep(t - now)
        tickets[i] = server.submit(q)
        ready[i].set()
    th.join()
    return np.asarray(lat), time.perf_counter() - t0


def fixed_load(duration_s: float = 3.0, rate: float = 200.0, m: int = 500_000, d: int = 50, k: int = 15,
               slots: int = 2, max_batch_cells: int = 65536, seed: int = 1) -> dict:
    """One replay of the serving workload at a fixed offered load: a seeded
    Poisson stream (`rate` requests/s for `duration_s`, query sizes
    log-uniform in [1, 20,000]) against an m x d atlas of 100 clusters.
    Returns p50/p99/mean latency (ms, submit to answer), answered cells/s,
    the service's counters (batches, most batches on the GPU at once, ...)
    and the workload's shape."""
    from . import synthetic

    atlas, centres = synthetic.serving_atlas(seed=0, m=m, d=d)
    times, counts = synthetic.poisson_arrivals(rate, duration_s, seed=seed)
    queries = [synthetic.serving_queries(centres, int(c), seed=100 + i) for i, c in enumerate(counts)]
    cells = int(counts.sum())
    with Server(atlas, k, slots=slots, max_batch_cells=max_batch_cells) as sv:
        sv.query(queries[0][:8])  # warm-up: workspaces and kernels
        lat, wall = _replay(sv, times, queries)
        st = sv.stats()
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "cells_per_s": cells / wall, "wall_s": wall,
            "requests": len(times), "query_cells": cells, "rate_per_s": rate, "duration_s": duration_s,
            "atlas_cells": m, "k": k, "slots": slots, "batches": st["batches"],
            "max_batches_in_flight": st["max_batches_in_flight"], "answered": st["requests"]}


def bench_main(args) -> int:
    """Serving workload: a 500,000 x 50 atlas (100 clusters) resident in HBM; Poisson arrivals
    at 200 requests/s; query sizes log-uniform in [1, 20,000]; k = 15 plus connectivity rows.
    Continuous batching (2 slots) against per-request launches (1 slot, one request per batch)."""
    from . import build

    build.build()
    m, d, k = 500_000, 50, 15
    rate, duration = 200.0, float(getattr(args, "serve_seconds", 0) or 5.0)
    result = {}
    for name, slots, max_cells in (("continuous", 2, 65536), ("per_request", 1, 1)):
        result[name] = fixed_load(duration, rate, m, d, k, slots=slots, max_batch_cells=max_cells)
    c = result["continuous"]
    line = {"metric": "serving p99 latency at 200 req/s (500k x 50 atlas, k = 15)", "value": c["p99_ms"],
            "unit": "ms", "n_gpus": 1, "steps": c["requests"], "warmup": 1, "ms_per_step": c["mean_ms"],
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f16", "data": "synthetic",
            "config": {"workload": "serving_500k_x50_k15", "atlas_cells": m, "dims": d, "k": k,
                       "rate_per_s": rate, "duration_s": duration, "requests": c["requests"],
                       "query_cells": c["query_cells"],
                       "query_sizes": "log-uniform [1, 20000], seed 1", "budget": "150 GiB"},
            "p50_ms": c["p50_ms"], "p99_ms": c["p99_ms"], "cells_per_s": c["cells_per_s"],
            "comparator": result["per_request"], "continuous": c}
    print(json.dumps(line), flush=True)
    return 0
