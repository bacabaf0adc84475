#!/usr/bin/env python
"""Throughput of the pp.neighbors graph build on GB300.

Workload (default): 1,000,000 cells x 50 dims f32, k = 15 non-self
neighbours, a seeded 200-cluster Gaussian mixture with 1% exact duplicates
(synthetic stand-in for a PCA embedding).  One step = kNN (exact, FP64-equal
neighbour lists) + the distances rows + UMAP connectivities CSR, on inputs
already resident in HBM.  `value` is cells/s over all ranks.  `e2e` is the
same through the host-pointer C-ABI call, with the embedding uploaded from
pinned memory and the kNN rows and connectivities CSR read back every step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--form plain|tensor]
    python bench.py --impl reference      # the reference CPU path (restated)

Outside the timed regions the default run also checks the bench graph
against the C oracle (10,000 random cells plus every zero-distance and
near-tie cell against the FP64 kNN; the whole connectivities CSR against the
restated connectivities), replays the serving workload at its fixed offered
load for its p50/p99 latency, and times the reference CPU path on a sample.

For N > 1 launch with torch.distributed.run; by default every rank builds its
own replica graph (no data-path collective, weak scaling); with
--parallelism sharded the ranks share one graph by rows (strong scaling).
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = {"name": "knn_graph_1M_x50_k15", "n": 1_000_000, "d": 50, "k": 15, "clusters": 200,
            "dup_frac": 0.01, "seed": 0}
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
# DRAM bytes of the sweep launches of one step at (n, d, k), from one ncu
# capture of this bench's own workload (dram__bytes_read.sum +
# dram__bytes_write.sum, a single-pass metric; profiles/tensor_sweep_1M_x50_k15.md):
# threshold pass 621.20 + 126.40 MB (its writes are the lists' register top-16),
# collect pass 734.45 + 122.71 MB.
SWEEP_TRAFFIC: dict = {(1_000_000, 50, 15): (621.20 + 126.40 + 734.45 + 122.71) * 1e6}
SWEEP_TRAFFIC_NOTE = ("bytes, dram__bytes_read.sum + dram__bytes_write.sum summed over the step's two sweep "
                      "launches (threshold pass, collect pass), one ncu capture of this workload")
FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--form", choices=["plain", "tensor"], default=None)
    p.add_argument("--n", type=int, default=WORKLOAD["n"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-recall", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--serve-seconds", type=float, default=3.0)
    p.add_argument("--parity-rows", type=int, default=10_000,
                   help="random cells checked against the FP64 oracle (plus every zero-distance and near-tie cell)")
    p.add_argument("--vs-plain", action="store_true", help="also solve with the plain form and compare")
    p.add_argument("--parallelism", choices=["replicas", "sharded"], default="replicas",
                   help="N > 1: independent replica graphs (weak scaling) or one graph sharded by rows (strong)")
    p.add_argument("--workload", choices=["precision", "batching", "serving", "scale"], default="precision",
                   help="precision: the 1M x 50 graph build (default); batching: 64 samples in one graph launch "
                        "against 64 sequential plain launches; serving: the resident-atlas query service; "
                        "scale: 100k x 50, k = 30, Euclidean and cosine")
    return p.parse_args()


def peaks():
    try:
        return json.loads(PEAKS_FILE.read_text()), "measured"
    except Exception:
        return FALLBACK_PEAKS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_data(n: int, seed: int):
    from mrustsc_gb300 import synthetic

    return synthetic.mixture(n, WORKLOAD["d"], clusters=WORKLOAD["clusters"], dup_frac=WORKLOAD["dup_frac"],
                             seed=seed)


# --------------------------------------------------------------------------- reference arm

def cpu_config(n: int) -> dict:
    """The GPU arm's config keys, so both arms name the same workload."""
    return {"workload": WORKLOAD["name"], "n_cells": n, "dims": WORKLOAD["d"], "k": WORKLOAD["k"],
            "clusters": WORKLOAD["clusters"], "dup_frac": WORKLOAD["dup_frac"], "mode": "exact"}


def cpu_reference_step(engine, k: int, rows: np.ndarray):
    """The reference CPU path (neighbors.rs:35-101 with its tile product on a
    BLAS SGEMM, as candle runs it) on a bounded sample: kNN of `rows` against
    all cells and the connectivities of that sample's graph (:208-372)."""
    from oracle import oracle

    idx, dist = engine.knn_rows(k, rows)
    sub = (idx % len(rows)).astype(np.uint32)
    oracle.connectivities(sub, dist)


def calibrate_rows(engine, k, seconds: float, n: int, cap: int = 200_000) -> np.ndarray:
    rng = np.random.default_rng(123)
    probe = np.sort(rng.choice(n, min(n, 2 * engine.tile_rows), replace=False))
    cpu_reference_step(engine, k, probe)  # first call: BLAS threads and buffers
    t0 = time.perf_counter()
    cpu_reference_step(engine, k, probe)
    per_row = (time.perf_counter() - t0) / len(probe)
    nrows = int(max(64, min(cap, n, seconds / max(per_row, 1e-9))))
    return np.sort(rng.choice(n, nrows, replace=False))


def cpu_sample_text(rows: int, n: int, secs: float, cores: int, engine) -> str:
    flop = 2.0 * rows * n * WORKLOAD["d"]
    return (f"{rows} query cells against all {n} (kNN + sample-graph connectivities) per step: the reference "
            f"CPU path restated (no Rust toolchain), tile product on numpy's BLAS SGEMM, affine/snap/selection "
            f"in C, {cores} threads; centring and norms once per workload, outside the steps; "
            f"{secs:.2f} s per step, {flop / secs / 1e9:.0f} GFLOP/s in the tile products")


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import oracle

    oracle.build()
    n, k = args.n, WORKLOAD["k"]
    x = make_data(n, WORKLOAD["seed"])
    engine = oracle.ExpansionCPU(x)
    step_seconds = min(10.0, max(2.0, 150.0 / max(1, args.steps + args.warmup)))
    rows = calibrate_rows(engine, k, step_seconds, n)
    for _ in range(args.warmup):
        cpu_reference_step(engine, k, rows)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cpu_reference_step(engine, k, rows)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * statistics.mean(times)
    value = len(rows) / (ms / 1e3)
    cores = oracle.num_threads()
    line = {"metric": "kNN-graph cells/s", "value": value, "unit": "cells/s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference", "config": cpu_config(n),
            "cpu_baseline": {"value": value, "unit": "cells/s", "cores": cores, "kind": "port",
                             "sample": cpu_sample_text(len(rows), n, ms / 1e3, cores, engine)},
            "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------- our arm

def parity_leg(torch, L, ctx, x, xd, k: int, form: str, idx_dev, dist_dev, n_random: int) -> tuple[dict, dict]:
    """The bench graph against the C oracle, outside every timed region: the
    kNN rows of `n_random` random cells plus every cell with a neighbour at
    distance 0 plus every cell whose k-th and (k+1)-th neighbours are within
    1e-5 relative (from one k+1 solve), against the FP64 exact kNN; and the
    whole connectivities CSR, built again through the host API, against the
    oracle's connectivities of the same kNN graph."""
    from mrustsc_gb300 import _scrust
    from oracle import oracle, parity

    oracle.build()
    n, d = x.shape
    st = _lib_status()
    i1 = torch.empty((n, k + 1), dtype=torch.int32, device=xd.device)
    d1 = torch.empty((n, k + 1), dtype=torch.float32, device=xd.device)
    opts = _lib_options(form)
    check(L.scrust_cuda_knn_device(ctx, xd.data_ptr(), n, d, k + 1, ctypes.byref(opts), i1.data_ptr(),
                                   d1.data_ptr(), ctypes.byref(st)), st)
    check(L.scrust_cuda_synchronize(ctx, ctypes.byref(st)), st)
    idx = idx_dev.cpu().numpy().view(np.uint32)
    dist = dist_dev.cpu().numpy()
    rows, kinds = parity.select_rows(n, dist, d1.cpu().numpy(), n_random=n_random, seed=0)
    t0 = time.perf_counter()
    rep = parity.knn_rows_report(x, k, idx, dist, rows)
    rep.update(kinds)
    rep["oracle_s"] = time.perf_counter() - t0
    rep["ok"] = parity.knn_rows_ok(rep)
    hi, hd, csr = _scrust.neighbors_graph(x, k, form=form)
    t0 = time.perf_counter()
    crep = parity.connectivities_report(hi, hd, csr)
    crep["oracle_s"] = time.perf_counter() - t0
    crep["knn_same_as_bench_graph"] = bool(np.array_equal(hi, idx) and np.array_equal(hd, dist))
    crep["ok"] = parity.connectivities_ok(crep) and crep["knn_same_as_bench_graph"]
    return rep, crep


def _lib_status():
    from mrustsc_gb300 import _lib

    return _lib.Status()


def _lib_options(form: str):
    from mrustsc_gb300 import _lib

    return _lib.options(form=form)


def check(rc, st):
    from mrustsc_gb300 import _lib

    _lib.check(rc, st)


def phase_bytes(form: str, n: int, d: int, k: int, nnz: int) -> dict:
    """Algorithmic bytes of the memory-bound phases: what each must read and
    write at least once.  prep: the embedding read, the candidate operands
    written (two n x 64 16-bit arrays in the tensor form, the transposed
    centred rows in the plain form); rerank: every row's coordinates read and
    the n x k ids and distances written; connectivities: the n x k graph read
    and the CSR (indptr, columns, values) written."""
    n_pad = (n + 255) // 256 * 256
    operands = 2 * n_pad * 64 * 2 if form == "tensor" else ((d + 3) // 4 * 4) * n_pad * 4
    return {"prep": n * d * 4 + operands, "rerank": n * d * 4 + n * k * 8,
            "connectivities": n * k * 8 + (n + 1) * 4 + nnz * 8}


def run_ours(args):
    import torch

    from mrustsc_gb300 import _lib, build

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    build.build()
    if args.parallelism == "sharded" and world > 1:
        return run_sharded(args, world, rank, local)
    L = _lib.lib()
    form = args.form or ("tensor" if getattr(_lib, "TENSOR_FORM_READY", False) else "plain")
    n, d, k = args.n, WORKLOAD["d"], WORKLOAD["k"]
    x = make_data(n, WORKLOAD["seed"] + rank)
    ctx = _lib.context(local)
    stream = torch.cuda.ExternalStream(L.scrust_cuda_context_stream(ctx))
    xd = torch.from_numpy(x).to(f"cuda:{local}")
    idx = torch.empty((n, k), dtype=torch.int32, device=xd.device)
    dst = torch.empty((n, k), dtype=torch.float32, device=xd.device)
    opts = _lib.options(form=form)
    st = _lib.Status()
    csr = ctypes.c_void_p()

    def step():
        rc = L.scrust_cuda_neighbors_graph_device(ctx, xd.data_ptr(), n, d, k, ctypes.byref(opts), idx.data_ptr(),
                                                  dst.data_ptr(), ctypes.byref(csr), ctypes.byref(st))
        _lib.check(rc, st)
        L.scrust_csr_free(csr)

    torch.cuda.synchronize()
    for _ in range(args.warmup):
        step()
    _lib.check(L.scrust_cuda_synchronize(ctx, ctypes.byref(st)), st)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()

    # Timed region: K steps, events on the library's stream; phase events on.
    L.scrust_cuda_set_timing(ctx, 1)
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = L.scrust_cuda_launch_count(ctx)
    phases = []
    buf = (ctypes.c_float * 8)()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    total_ms = 0.0
    for _ in range(args.steps):
        start.record(stream)
        step()
        end.record(stream)
        end.synchronize()
        total_ms += start.elapsed_time(end)
        got = L.scrust_cuda_phase_times(ctx, buf, 8)
        phases.append([buf[i] for i in range(got)])
    torch.cuda.synchronize()
    launches = int(L.scrust_cuda_launch_count(ctx) - launches0)
    clk = clocks.stop()
    L.scrust_cuda_set_timing(ctx, 0)
    _lib.check(L.scrust_cuda_synchronize(ctx, ctypes.byref(st)), st)
    ms_step = total_ms / args.steps
    if world > 1:
        t = torch.tensor([ms_step], device=xd.device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_step = float(t.item())
        torch.distributed.barrier()
    value = world * n / (ms_step / 1e3)

    # One more (untimed) step for the graph's size.
    out = ctypes.c_void_p()
    _lib.check(L.scrust_cuda_neighbors_graph_device(ctx, xd.data_ptr(), n, d, k, ctypes.byref(opts), idx.data_ptr(),
                                                    dst.data_ptr(), ctypes.byref(out), ctypes.byref(st)), st)
    nnz = int(L.scrust_csr_nnz(out))
    L.scrust_csr_free(out)

    ph = np.array(phases) if phases and len(phases[0]) == 8 else np.zeros((1, 8))
    ph_mean = ph.mean(0)
    cand_ms = float(ph_mean[1])
    pk, pk_kind = peaks()
    hbm = float(pk["hbm_gbs"])
    if form == "tensor":
        # The dominant kernel is the tensor sweep (knn_candidates_tc): its
        # passes are timed by the library's events on its stream (the
        # candidates phase less the building of the second pass's tile
        # lists).  Its unit of work is one (256-row block, 256-column tile)
        # pair, 2 * 256 * 256 * d algorithmic flops; the pairs it computes are
        # counted by the kernel's own counters in one extra, untimed step.
        sweep_ms = cand_ms - float(ph_mean[5]) if ph_mean[4] > 0 else cand_ms
        cnt = (ctypes.c_uint64 * 80)()
        L.scrust_cuda_kernel_stats(ctx, 1, cnt, 80)
        step()
        _lib.check(L.scrust_cuda_synchronize(ctx, ctypes.byref(st)), st)
        L.scrust_cuda_kernel_stats(ctx, 0, cnt, 80)
        tiles = int(cnt[8])
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        if ph_mean[4] > 0:
            # The launches of an ordered solve (k <= 32), with their own
            # counters: the threshold pass over the priority tiles, then one
            # collect pass over the priority tiles and the tiles the tile
            # balls keep.
            pass_ms = [float(ph_mean[4]), float(ph_mean[7])]
            names = ["threshold, priority tiles", "collect, priority and kept tiles"]
            sweep_passes = []
            for i, name in enumerate(names):
                c = [int(cnt[16 * (i + 1) + j]) for j in range(16)]
                t = c[8]
                sweep_passes.append({"pass": name, "ms": pass_ms[i], "tiles": t,
                                     "us_per_tile_per_sm": pass_ms[i] * 1e3 * sms / t if t else None,
                                     "appends": c[0], "topk_chunks_entered": c[12], "topk_bulk_merges": c[13],
                                     "topk_insert_rounds": c[14], "topk_entrants": c[15]})
        blocks = (n + 255) // 256
        flops = tiles * 2.0 * 256 * 256 * d
        achieved = flops / (sweep_ms / 1e3) / 1e12
        traffic = SWEEP_TRAFFIC.get((n, d, k))
        roof = {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                "frac": achieved / pk["bf16_tflops"], "traffic": traffic,
                "traffic_note": SWEEP_TRAFFIC_NOTE if traffic else None,
                "kernel": "tensor_candidates_kernel (knn_candidates_tc), all sweep passes",
                "kernel_ms": sweep_ms, "units": "(256-row block, 256-column tile) pairs computed",
                "units_per_step": tiles, "flops_per_unit": 2 * 256 * 256 * d,
                "brute_force_units": blocks * blocks, "peak_source": f"bf16 burst, {pk_kind}"}
        if ph_mean[4] > 0:
            roof["passes"] = sweep_passes
    else:
        flops = 2.0 * n * n * d
        sm_count = torch.cuda.get_device_properties(local).multi_processor_count
        fp32_peak = sm_count * 128 * 2 * float(pk.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
        achieved = flops / (cand_ms / 1e3) / 1e12
        roof = {"bound": "fp32_cuda_core", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak, "traffic": None, "kernel": "plain_candidates_kernel",
                "peak_source": f"{sm_count} SMs x 128 FP32 lanes x 2 x {pk.get('sm_max_mhz', 2070.0)} MHz"}
    pb = phase_bytes(form, n, d, k, nnz)
    phase_ms = {"prep": float(ph_mean[0]), "rerank": float(ph_mean[2]), "connectivities": float(ph_mean[3])}
    phases_gbs = {name: {"bytes": pb[name], "ms": phase_ms[name],
                         "gbs": pb[name] / (phase_ms[name] / 1e3) / 1e9 if phase_ms[name] > 0 else None,
                         "frac_of_hbm": (pb[name] / (phase_ms[name] / 1e3) / 1e9) / hbm if phase_ms[name] > 0 else None}
                  for name in phase_ms}

    line = {"metric": "kNN-graph cells/s", "value": value, "unit": "cells/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if form == "plain" else "f16",
            "data": "synthetic",
            "config": {**cpu_config(n), "form": form, "parallelism": f"replicas{world}",
                       "l2": "inputs larger than L2 (200 MB embedding, >1 GB candidate lists per step)"},
            "phases_ms": {"prep": float(ph_mean[0]), "candidates": float(ph_mean[1]),
                          "rerank": float(ph_mean[2]), "connectivities": float(ph_mean[3]),
                          "candidates_first_pass": float(ph_mean[4]),
                          "candidates_tile_lists": float(ph_mean[5]),
                          "candidates_collect": float(ph_mean[7])},
            "phases_gbs": phases_gbs, "phases_gbs_peak": f"{hbm} GB/s, {pk_kind} copy bandwidth",
            "graph_nnz": nnz, "gpu_launches": launches, "roofline": roof, "clocks": clk}

    if rank == 0 and not args.no_e2e:
        # Pinned host buffers for the input and both neighbour arrays (the
        # graph's host arrays come from the library's own pinned pool).  The
        # same K steps as the device-resident timing, each one call of the
        # host API: upload, graph, download of the kNN rows and the CSR.
        # Timed before the parity leg, whose multi-threaded oracle would
        # otherwise still hold the host cores the call's thread waits on.
        xh = torch.from_numpy(x).pin_memory()
        ih = torch.empty((n, k), dtype=torch.int32).pin_memory()
        dh = torch.empty((n, k), dtype=torch.float32).pin_memory()
        e2e_steps = max(1, args.steps)
        nnz_e = 0
        # W untimed calls first (at least one): they size the device
        # workspaces and the pinned pool, as the warm-up steps do for the
        # device-resident timing.
        for _ in range(max(1, args.warmup)):
            out = ctypes.c_void_p()
            _lib.check(L.scrust_cuda_neighbors_graph(ctx, xh.data_ptr(), n, d, k, ctypes.byref(opts), ih.data_ptr(),
                                                     dh.data_ptr(), ctypes.byref(out), ctypes.byref(st)), st)
            L.scrust_csr_free(out)
        times = []
        for _ in range(e2e_steps):
            t0 = time.perf_counter()
            out = ctypes.c_void_p()
            rc = L.scrust_cuda_neighbors_graph(ctx, xh.data_ptr(), n, d, k, ctypes.byref(opts), ih.data_ptr(),
                                               dh.data_ptr(), ctypes.byref(out), ctypes.byref(st))
            _lib.check(rc, st)
            times.append(time.perf_counter() - t0)
            nnz_e = int(L.scrust_csr_nnz(out))
            L.scrust_csr_free(out)
        e2e_s = statistics.mean(times)
        line["e2e"] = {"value": n / e2e_s, "unit": "cells/s", "h2d_bytes_per_step": n * d * 4,
                       "d2h_bytes_per_step": n * k * 8 + (n + 1) * 4 + nnz_e * 8, "ms_per_step": e2e_s * 1e3,
                       "steps": e2e_steps, "ms_min": min(times) * 1e3, "ms_max": max(times) * 1e3}

    if rank == 0 and not args.no_recall:
        rep, crep = parity_leg(torch, L, ctx, x, xd, k, form, idx, dst, args.parity_rows)
        line["recall_fp64_sample"] = rep
        line["conn_check"] = crep
        if form == "tensor" and args.vs_plain:
            idx_t = idx.clone()
            opts_p = _lib.options(form="plain")
            rc = L.scrust_cuda_knn_device(ctx, xd.data_ptr(), n, d, k, ctypes.byref(opts_p), idx.data_ptr(),
                                          dst.data_ptr(), ctypes.byref(st))
            _lib.check(rc, st)
            torch.cuda.synchronize()
            line["recall_vs_plain"] = float((idx_t == idx).all(1).float().mean().item())

    if rank == 0 and world == 1 and not args.no_serving and args.n == WORKLOAD["n"]:
        from mrustsc_gb300 import serving

        line["serving"] = serving.fixed_load(duration_s=args.serve_seconds)

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle

        oracle.build()
        engine = oracle.ExpansionCPU(x)
        rows = calibrate_rows(engine, k, args.cpu_seconds, n)
        t0 = time.perf_counter()
        cpu_reference_step(engine, k, rows)
        secs = time.perf_counter() - t0
        cores = oracle.num_threads()
        line["cpu_baseline"] = {"value": len(rows) / secs, "unit": "cells/s", "cores": cores, "kind": "port",
                                "sample": cpu_sample_text(len(rows), n, secs, cores, engine)}
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_sharded(args, world: int, rank: int, local: int):
    """One graph sharded over the ranks (strong scaling): each rank solves its
    block of rows against the whole embedding on its GPU, the rows are
    gathered into device tensors with NCCL, and rank 0 builds the
    connectivities.  A step ends when rank 0's graph is complete."""
    import torch
    import torch.distributed as dist

    from mrustsc_gb300 import _lib, distributed

    L = _lib.lib()
    n, d, k = args.n, WORKLOAD["d"], WORKLOAD["k"]
    x = make_data(n, WORKLOAD["seed"])
    xd = torch.from_numpy(x).to(f"cuda:{local}")

    def step():
        res = distributed.neighbors_sharded_device(xd, k, rank, world)
        if res[2] is not None:
            _lib.check(L.scrust_cuda_synchronize(_lib.context(local), ctypes.byref(_lib.Status())), _lib.Status())
            L.scrust_csr_free(res[2])

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    end.record()
    end.synchronize()
    clk = clocks.stop()
    t = torch.tensor([start.elapsed_time(end) / args.steps], device=xd.device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_step = float(t.item())
    dist.barrier()
    dist.destroy_process_group()
    if rank == 0:
        line = {"metric": "kNN-graph cells/s", "value": n / (ms_step / 1e3), "unit": "cells/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
                "scaling": "strong", "vs_baseline": None, "dtype": "f16", "data": "synthetic",
                "config": {**cpu_config(n), "form": "tensor", "parallelism": f"sharded{world}",
                           "l2": "inputs larger than L2"},
                "clocks": clk}
        print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------- batching

def run_batching(args):
    """64 samples (sizes log-uniform in [500, 50,000], 4-20 clusters each, k = 15): every sample's graph
    (kNN + UMAP connectivities) in one CUDA-graph launch of the batched tensor sweep and the batch's
    fuzzy union, against the kNN-only plan, 64 sequential plain launches and 64 sequential tensor
    launches on the same data."""
    import torch

    from mrustsc_gb300 import _lib, build, synthetic

    build.build()
    L = _lib.lib()
    k, d = 15, 50
    samples = synthetic.batch_samples(seed=0)
    sizes = [len(x) for x in samples]
    x = np.concatenate(samples)
    n = len(x)
    offsets = np.zeros(len(samples) + 1, dtype=np.uint64)
    offsets[1:] = np.cumsum(sizes)
    ctx = _lib.context(0)
    stream = torch.cuda.ExternalStream(L.scrust_cuda_context_stream(ctx))
    xd = torch.from_numpy(x).cuda()
    idx = torch.empty((n, k), dtype=torch.int32, device="cuda")
    dst = torch.empty((n, k), dtype=torch.float32, device="cuda")
    gidx = torch.empty((n, k), dtype=torch.int32, device="cuda")
    gdst = torch.empty((n, k), dtype=torch.float32, device="cuda")
    st = _lib.Status()
    opts = _lib.options(form="tensor")
    t0 = time.perf_counter()
    gplan = L.scrust_cuda_batch_plan_create_graphs(ctx, _lib.ptr(offsets), len(samples), d, k, ctypes.byref(opts),
                                                   xd.data_ptr(), gidx.data_ptr(), gdst.data_ptr(), ctypes.byref(st))
    if not gplan:
        raise RuntimeError(st.message.decode())
    plan_s = time.perf_counter() - t0
    plan = L.scrust_cuda_batch_plan_create(ctx, _lib.ptr(offsets), len(samples), d, k, ctypes.byref(opts),
                                           xd.data_ptr(), idx.data_ptr(), dst.data_ptr(), ctypes.byref(st))
    if not plan:
        raise RuntimeError(st.message.decode())
    cap, prec, tuned = ctypes.c_uint32(), ctypes.c_int32(), ctypes.c_float()
    L.scrust_cuda_batch_plan_choice(gplan, ctypes.byref(cap), ctypes.byref(prec), ctypes.byref(tuned))
    width = int(L.scrust_cuda_batch_plan_topk_width(gplan))

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / steps

    clocks = ClockSampler(0)
    clocks.start()
    launches0 = L.scrust_cuda_launch_count(ctx)
    ms_graphs = timed(lambda: _lib.check(L.scrust_cuda_batch_plan_launch(gplan, ctypes.byref(st)), st),
                      args.steps, args.warmup)
    launches = int(L.scrust_cuda_launch_count(ctx) - launches0)
    clk = clocks.stop()
    ms_knn = timed(lambda: _lib.check(L.scrust_cuda_batch_plan_launch(plan, ctypes.byref(st)), st),
                   args.steps, args.warmup)
    _lib.check(L.scrust_cuda_synchronize(ctx, ctypes.byref(st)), st)
    # The graph plan's CSR, read through the CUDA array interface.
    ip, ix, vl = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    L.scrust_cuda_batch_plan_graph(gplan, ctypes.byref(ip), ctypes.byref(ix), ctypes.byref(vl))

    class DeviceView:
        def __init__(self, ptr, count, typestr):
            self.__cuda_array_interface__ = {"shape": (count,), "typestr": typestr, "data": (ptr, False),
                                             "version": 2}

    def grab(ptr, count, typestr):
        return torch.as_tensor(DeviceView(ptr.value, count, typestr), device="cuda").cpu().numpy()

    indptr = grab(ip, n + 1, "<u4")
    nnz = int(indptr[-1])
    cols, vals = grab(ix, nnz, "<u4"), grab(vl, nnz, "<f4")
    graph_idx = gidx.clone()
    graph_dist = gdst.clone()

    plain = _lib.options(form="plain")
    views = [(xd[int(offsets[s]):int(offsets[s + 1])], idx[int(offsets[s]):int(offsets[s + 1])],
              dst[int(offsets[s]):int(offsets[s + 1])]) for s in range(len(samples))]

    def sequential(o):
        def run():
            for xs, ii, dd in views:
                _lib.check(L.scrust_cuda_knn_device(ctx, xs.data_ptr(), len(xs), d, k, ctypes.byref(o),
                                                    ii.data_ptr(), dd.data_ptr(), ctypes.byref(st)), st)
        return run

    seq_steps = max(1, min(args.steps, 3))
    ms_plain = timed(sequential(plain), seq_steps, 1)
    same = bool((graph_idx == idx).all().item())
    ms_tensor_seq = timed(sequential(opts), seq_steps, 1)
    L.scrust_cuda_batch_plan_destroy(plan)
    L.scrust_cuda_batch_plan_destroy(gplan)

    # e2e through the host-pointer batch graph call: upload, graphs, download of
    # the kNN rows and the CSR, from and into pinned host buffers (one untimed
    # call first, as for the main e2e).
    ih = torch.empty((n, k), dtype=torch.int32).pin_memory()
    dh = torch.empty((n, k), dtype=torch.float32).pin_memory()
    xh = torch.from_numpy(np.ascontiguousarray(x)).pin_memory()
    e2e_steps = max(1, args.steps)
    e2e_nnz = 0
    times = []
    for it in range(e2e_steps + 1):
        t0 = time.perf_counter()
        out = ctypes.c_void_p()
        _lib.check(L.scrust_cuda_neighbors_graph_batch(ctx, xh.data_ptr(), _lib.ptr(offsets), len(samples), d, k,
                                                       ctypes.byref(opts), ih.data_ptr(), dh.data_ptr(),
                                                       ctypes.byref(out), ctypes.byref(st)), st)
        e2e_nnz = int(L.scrust_csr_nnz(out))
        L.scrust_csr_free(out)
        if it:
            times.append(time.perf_counter() - t0)
    e2e_s = statistics.mean(times)
    flops = sum(2.0 * m * m * d for m in sizes)
    parity_rep = conn_rep = None
    if not args.no_recall:
        # Every sample: 64 random rows and up to 64 rows with a zero-distance
        # neighbour against the FP64 kNN of that sample, and the sample's whole
        # CSR against the restated connectivities of its kNN graph (outside
        # the timing).
        from mrustsc_gb300._scrust import split_batch_graph
        from oracle import oracle, parity

        oracle.build()
        gi = graph_idx.cpu().numpy().view(np.uint32)
        gd = graph_dist.cpu().numpy()
        rng = np.random.default_rng(1)
        rows_total, exact, worst = 0, 0, 0.0
        c_ok, c_err = 0, 0.0
        for s_i, (xs, (si, sd, csr)) in enumerate(zip(samples, split_batch_graph(offsets, gi, gd, indptr, cols,
                                                                                 vals))):
            rows = np.unique(np.concatenate([rng.choice(len(xs), min(len(xs), 64), replace=False),
                                             np.nonzero(sd[:, 0] == 0)[0][:64]]))
            rep = parity.knn_rows_report(xs, k, si, sd, rows)
            rows_total += rep["rows"]
            exact += rep["exact_rows"]
            worst = max(worst, rep["max_rel_dist_err"])
            crep = parity.connectivities_report(si, sd, csr)
            c_ok += int(parity.connectivities_ok(crep))
            c_err = max(c_err, crep["max_abs_err"] or float("inf"))
        parity_rep = {"samples": len(samples), "rows": rows_total, "exact_rows": exact, "max_rel_dist_err": worst,
                      "against": "FP64 exact kNN of each sample (C oracle)"}
        conn_rep = {"samples": len(samples), "samples_equal": c_ok, "max_abs_err": c_err, "nnz": nnz,
                    "against": "restated connectivities of each sample's kNN graph (C oracle)"}
    line = {"metric": "batched kNN-graph cells/s (64 samples, kNN + connectivities, one CUDA-graph launch)",
            "value": n / (ms_graphs / 1e3), "unit": "cells/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_graphs, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f16" if prec.value == 0 else "bf16", "data": "synthetic",
            "config": {"workload": "batching_64_samples_k15", "samples": len(samples), "cells": n, "dims": d, "k": k,
                       "sizes": "log-uniform [500, 50000], seed 0", "sum_2n2d_flop": flops,
                       "l2": "inputs and lists larger than L2"},
            "comparator": {"knn_only_plan_ms": ms_knn, "graphs_over_knn_only": ms_graphs / ms_knn,
                           "sequential_plain_knn_ms": ms_plain, "sequential_tensor_knn_ms": ms_tensor_seq,
                           "speedup_vs_sequential_plain": ms_plain / ms_graphs,
                           "knn_identical_to_sequential_plain": same},
            "autotuner": {"list_capacity": cap.value, "topk_width": width,
                          "precision": "fp16" if prec.value == 0 else "bf16", "tuned_ms": tuned.value,
                          "plan_create_s": plan_s,
                          "fixed": "tile shape (2 x 128-row MMA halves x 256-column tiles, K = 64)"},
            "gpu_launches": launches, "clocks": clk, "recall_fp64_sample": parity_rep, "conn_check": conn_rep,
            "e2e": {"value": n / e2e_s, "unit": "cells/s", "h2d_bytes_per_step": n * d * 4,
                    "d2h_bytes_per_step": n * k * 8 + (n + 1) * 4 + e2e_nnz * 8, "ms_per_step": e2e_s * 1e3,
                    "steps": e2e_steps}}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------- plain scale (100k, k = 30)

def run_scale(args):
    """100,000 x 50, k = 30, 40 clusters, 0.5% duplicates and 0.5% near-duplicates: the graph build
    (kNN + connectivities) for the Euclidean and the cosine metric, plain and tensor forms."""
    import torch

    from mrustsc_gb300 import _lib, build, synthetic

    build.build()
    L = _lib.lib()
    n, d, k = 100_000, 50, 30
    x = synthetic.plain_scale(seed=0, n=n)
    ctx = _lib.context(0)
    stream = torch.cuda.ExternalStream(L.scrust_cuda_context_stream(ctx))
    xd = torch.from_numpy(x).cuda()
    idx = torch.empty((n, k), dtype=torch.int32, device="cuda")
    dst = torch.empty((n, k), dtype=torch.float32, device="cuda")
    st = _lib.Status()
    csr = ctypes.c_void_p()
    res = {}
    clocks = ClockSampler(0)
    clocks.start()
    for metric in ("euclidean", "cosine"):
        outs = {}
        for form in ("plain", "tensor"):
            o = _lib.options(form=form, metric=metric)

            def step():
                _lib.check(L.scrust_cuda_neighbors_graph_device(ctx, xd.data_ptr(), n, d, k, ctypes.byref(o),
                                                                idx.data_ptr(), dst.data_ptr(), ctypes.byref(csr),
                                                                ctypes.byref(st)), st)
                L.scrust_csr_free(csr)

            for _ in range(args.warmup):
                step()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            steps = max(1, min(args.steps, 10))
            a.record(stream)
            for _ in range(steps):
                step()
            b.record(stream)
            b.synchronize()
            ms = a.elapsed_time(b) / steps
            outs[form] = idx.clone()
            res[f"{metric}_{form}"] = {"cells_per_s": n / (ms / 1e3), "ms_per_step": ms}
        res[f"{metric}_forms_identical"] = bool((outs["plain"] == outs["tensor"]).all().item())
    clk = clocks.stop()
    best = res["euclidean_tensor"]
    line = {"metric": "kNN-graph cells/s at 100k x 50, k = 30", "value": best["cells_per_s"], "unit": "cells/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": best["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f16", "data": "synthetic",
            "config": {"workload": "plain_scale_100k_x50_k30", "n_cells": n, "dims": d, "k": k, "clusters": 40,
                       "dup_frac": 0.005, "near_dup_frac": 0.005},
            "results": res, "clocks": clk}
    print(json.dumps(line), flush=True)
    return 0


def run_serving(args):
    from mrustsc_gb300 import serving

    return serving.bench_main(args)


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batching":
        return run_batching(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "scale":
        return run_scale(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
