"""Benchmark: boosting trees/s on the 10M x 128 regression workload on GB300.

Workload (the reference project's large regression configuration): 10,000,000 rows x 128
float32 features (64 N(0,1), 32 lognormal(0,1), 32 uniform integers in [0,1000)),
y = sum of 16 seeded random pairwise feature products + N(0, 0.5), sample weights
U(0.5, 1.5); quantile binning to 255 bins; depth 8, learning rate 0.05, squared error,
min_samples_leaf 20, min_child_weight 1, reg_lambda 1. A step is one boosting round
(one tree). Data are seeded synthetic inputs of that shape and distribution.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --only-train [--rows R] [--max-bins B] [--no-autotune]   (rounds only)
  python bench.py --workload logistic | forest                            (other configurations)

Our arm prints one JSON line with the whole-job trees/s measured with CUDA events on the
backend stream (inputs resident in HBM), an end-to-end figure through the C ABI from
pinned host buffers, the histogram kernel's roofline and a CPU baseline (the oracle's
restatement of the reference trainer on host cores, on a bounded row sample scaled to the
full workload). ``--impl reference`` times that CPU implementation alone.
Under torchrun each rank trains an independent replica on its own GPU.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ROWS, FEATURES, BINS, DEPTH, LR, TREES = 10_000_000, 128, 255, 8, 0.05, 200
SEED = 20260719 + 2
PARAMS = dict(max_depth=DEPTH, learning_rate=LR, min_samples_leaf=20, min_child_weight=1.0,
              reg_lambda=1.0, max_bins=BINS)
METRIC = "trees/s @10Mx128x255bins d8 (fixed-point batched)"
# DRAM traffic of the histogram launches per algorithmic byte: one ncu capture of
# dram__bytes_read.sum + dram__bytes_write.sum over the eight histogram launches of a
# steady-state round of this workload at 4M rows (2,219.7 MB against 1,958.3 MB), recorded
# with its command in the profile named below; scaled by the live algorithmic bytes.
HIST_TRAFFIC_PER_ALG_BYTE = 1.133
HIST_TRAFFIC_PROFILE = "profiles/hist_build_dram_traffic_10Mx128_d8.md"
CONFIG = {
    "workload": "regression 10,000,000 rows x 128 features (64 normal, 32 lognormal, 32 int[0,1000)), "
                "255 bins, depth 8, lr 0.05, weighted squared error",
    "rows": ROWS, "features": FEATURES, "bins": BINS, "max_depth": DEPTH, "learning_rate": LR,
    "n_estimators": TREES,
    "hist": "int64 fixed-point, all frontier nodes per launch, one CUDA graph per round",
    "l2": "inputs (1.28 GB binned matrix) exceed the 129 MB L2; no flush between steps",
}


def make_data(rows: int, seed: int = SEED):
    """Feature-major float32 matrix [features, rows], labels, weights."""
    rng = np.random.default_rng(seed)
    xf = np.empty((FEATURES, rows), np.float32)
    for f in range(64):
        xf[f] = rng.standard_normal(rows, dtype=np.float32)
    for f in range(64, 96):
        xf[f] = np.exp(rng.standard_normal(rows, dtype=np.float32))
    for f in range(96, 128):
        xf[f] = rng.integers(0, 1000, rows).astype(np.float32)
    pairs = rng.choice(FEATURES, size=(16, 2))
    scale = np.ones(FEATURES, np.float32)
    scale[64:96] = 1.0 / 1.65  # lognormal mean
    scale[96:] = 1.0 / 500.0
    y = rng.normal(0.0, 0.5, rows)
    for a, b in pairs:
        y += (xf[a] * scale[a]).astype(np.float64) * (xf[b] * scale[b])
    w = rng.uniform(0.5, 1.5, rows)
    return xf, y, w


def make_logistic_data(rows: int = 4_000_000):
    """Binary logistic configuration: rows x 256 float32 (200 N(0,1) features and 56
    integer features with 2-16 distinct values), 10 % of all cells NaN; labels ~
    Bernoulli(sigmoid(w . x[:32] + 0.5 x0 x1)), w ~ N(0, 1/32), missing cells read as 0
    in the label model. Row-major [rows, 256]."""
    f_cont, f_int = 200, 56
    rng = np.random.default_rng(20260719 + 3)
    x = np.empty((rows, f_cont + f_int), np.float32)
    x[:, :f_cont] = rng.standard_normal((rows, f_cont), dtype=np.float32)
    card = rng.integers(2, 17, f_int)
    for j in range(f_int):
        x[:, f_cont + j] = rng.integers(0, card[j], rows)
    for lo in range(0, f_cont + f_int, 32):  # 10 % NaN, a column block at a time
        blk = x[:, lo:lo + 32]
        blk[rng.random(blk.shape, dtype=np.float32) < 0.1] = np.nan
    xs = np.nan_to_num(x[:, :32]).astype(np.float64)
    logit = xs @ rng.normal(0.0, np.sqrt(1.0 / 32), 32) + 0.5 * xs[:, 0] * xs[:, 1]
    y = (rng.random(rows) < 1.0 / (1.0 + np.exp(-logit))).astype(np.float64)
    return x, y


def make_ovr_data(rows: int = 2_000_000, features: int = 64, classes: int = 10):
    """One-vs-rest configuration: rows x 64 N(0,1) float32; class = argmax of 10 random
    linear scores plus Gumbel noise."""
    rng = np.random.default_rng(20260719 + 4)
    x = rng.standard_normal((rows, features), dtype=np.float32)
    scores = x @ rng.standard_normal((features, classes), dtype=np.float32)
    scores += rng.gumbel(size=(rows, classes)).astype(np.float32)
    return x, scores.argmax(axis=1).astype(np.float64)


def make_forest_data(rows: int = 1_000_000, features: int = 100, trees: int = 256):
    """Random-forest configuration: rows x 100 N(0,1) float32, Friedman-1 target on
    x0..x4 (scaled to [0, 1]) + N(0,1); per tree Poisson(1) row counts and a sorted
    subset of 10 = sqrt(100) features."""
    rng = np.random.default_rng(20260719 + 5)
    x = rng.standard_normal((rows, features), dtype=np.float32)
    u = (x[:, :5] - x[:, :5].min(0)) / (x[:, :5].max(0) - x[:, :5].min(0))
    y = (10 * np.sin(np.pi * u[:, 0] * u[:, 1]) + 20 * (u[:, 2] - 0.5) ** 2 + 10 * u[:, 3] + 5 * u[:, 4]
         + rng.normal(size=rows))
    counts = rng.poisson(1.0, size=(trees, rows)).astype(np.uint8)
    subsets = [np.sort(rng.choice(features, size=10, replace=False)) for _ in range(trees)]
    return x, y, counts, subsets


def sample_clocks(stop: threading.Event, out: list):
    cmd = ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
           "--format=csv,noheader,nounits"]
    dev = os.environ.get("LOCAL_RANK", "0")
    while not stop.is_set():
        try:
            line = subprocess.run(cmd + ["-i", dev], capture_output=True, text=True, timeout=5).stdout.strip()
            if line:
                out.append([v.strip() for v in line.split(",")])
        except Exception:
            pass
        stop.wait(0.2)


def clocks_summary(samples):
    if not samples:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
    sm = [float(s[1]) for s in samples if s[1].replace(".", "").isdigit()]
    mx = [float(s[2]) for s in samples if s[2].replace(".", "").isdigit()]
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    reasons = sorted({names[i] for s in samples for i in range(4) if len(s) > 4 + i and s[4 + i] == "Active"})
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons, "samples": len(samples)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_baseline(xf, y, w, sample_rows: int, trees: int):
    """The oracle's FP64 restatement of the reference trainer on a leading row sample,
    on one core as the reference trainer runs."""
    import oracle

    oracle.build(reference=False)
    orc = oracle.Oracle("port")
    orc.set_threads(1)
    x = xf[:, :sample_rows].T  # strided view, columns contiguous
    t0 = time.perf_counter()
    ds = orc.quantize_dense(x, BINS)
    tq = time.perf_counter() - t0
    t0 = time.perf_counter()
    orc.train_regressor(ds, y[:sample_rows], w[:sample_rows], hist_mode=oracle.HIST_FP64,
                        n_estimators=trees, **PARAMS)
    dt = time.perf_counter() - t0
    per_tree_full = dt / trees * (ROWS / sample_rows)
    return {
        "value": 1.0 / per_tree_full, "unit": "trees/s", "cores": 1, "kind": "port",
        "note": "the reference's own trainer, compiled from its sources on x86 host cores, ran "
                "2.1x slower than this port on 200,000 x 128 rows, depth 8, with identical trees",
        "sample": f"{trees} tree(s) on the first {sample_rows:,} rows ({dt:.1f} s training, "
                  f"{tq:.1f} s binning), time per tree scaled by rows to {ROWS:,}",
    }


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return rank, world


def reduce_max(value: float, world: int) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def run_reference(args, rank, world):
    if rank != 0:
        return
    xf, y, w = make_data(args.ref_rows)
    import oracle

    oracle.build(reference=False)
    orc = oracle.Oracle("port")
    orc.set_threads(1)  # the reference trainer is single-threaded
    ds = orc.quantize_dense(xf.T, BINS)
    warm = max(1, min(args.warmup, 3))
    orc.train_regressor(ds, y, w, hist_mode=oracle.HIST_FP64, n_estimators=warm, **PARAMS)
    t0 = time.perf_counter()
    orc.train_regressor(ds, y, w, hist_mode=oracle.HIST_FP64, n_estimators=args.steps, **PARAMS)
    dt = time.perf_counter() - t0
    value = args.steps / dt * (args.ref_rows / ROWS)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "trees/s", "n_gpus": world,
        "steps": args.steps, "warmup": warm, "ms_per_step": dt / args.steps * 1e3 * (ROWS / args.ref_rows),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": CONFIG,
        "cpu_baseline": {"value": value, "unit": "trees/s", "cores": 1, "kind": "port",
                         "sample": f"each step one tree on the first {args.ref_rows:,} rows, "
                                   f"time scaled by rows to {ROWS:,} (single-threaded, as the reference)"},
        "e2e": {"value": value, "unit": "trees/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world):
    import mpsboost_gb300 as mb
    from mpsboost_gb300 import _lib

    local = int(os.environ.get("LOCAL_RANK", "0"))
    xf, y, w = make_data(args.rows)
    t0 = time.perf_counter()
    binned = mb.quantize_dense(xf.T, args.max_bins)
    t_bin = time.perf_counter() - t0
    params = dict(PARAMS, max_bins=args.max_bins)
    backend = mb.CudaBackend(local)
    # The same binning on the device (QuantizeDense on the GPU), host matrix to resident
    # bins; checked against the host bins.
    mb.quantize_device(backend, xf[:, :1024].T, args.max_bins).close()  # warm the kernels
    backend.synchronize()
    t0 = time.perf_counter()
    dbin = mb.quantize_device(backend, xf.T, args.max_bins)
    backend.synchronize()
    t_dbin = time.perf_counter() - t0
    dbin_equal = bool(np.array_equal(dbin.bin_counts, binned.bin_counts))
    dbin.close()
    # Launch shape for this fit shape: the autotuner times rounds under candidate shapes and
    # every later session below (timed, roofline, end to end) uses the fastest.
    tuning = (backend.autotune(binned, y, w, rounds_per_trial=5, **params) if not args.no_autotune
              else {"hist_threads": 768, "hist_stages": 2, "root_threads": 1024, "items_per_sm": 3,
                    "blocked_levels": 2, "scan_threads": 128, "trials": 0, "ms_per_round": 0.0,
                    "default_ms_per_round": 0.0})
    n_rounds = args.warmup + args.steps
    trainer = mb.Trainer(backend, binned, y, w, n_estimators=2 * n_rounds + 4, **params)
    trainer.run(args.warmup)
    trainer.synchronize()
    trainer.reset_stats()

    # Timed region: K rounds, CUDA events on the backend stream.
    samples: list = []
    stop = threading.Event()
    sampler = threading.Thread(target=sample_clocks, args=(stop, samples), daemon=True)
    sampler.start()
    barrier(world)
    backend.synchronize()
    backend.timer_begin()
    trainer.run(args.steps)
    ms = backend.timer_end()
    backend.synchronize()
    barrier(world)
    stop.set()
    sampler.join()
    trainer.synchronize()
    st = trainer.stats()
    ms_max = reduce_max(ms, world)
    value = world * args.steps / (ms_max / 1e3)
    if args.only_train:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "trees/s", "rows": args.rows,
                              "max_bins": args.max_bins,
                              "steps": args.steps, "warmup": args.warmup,
                              "gpu_launches": int(st["kernel_launches"]), "only_train": True,
                              "hist_cells": int(st["hist_cells"]), "hist_rows": int(st["hist_rows"]),
                              "part_rows": int(st["part_rows"])}),
                  flush=True)
        trainer.close()
        return

    # Roofline pass: the same rounds with CUDA events around every histogram launch.
    timed = mb.Trainer(backend, binned, y, w, n_estimators=n_rounds, options=_lib.OPT_TIMING, **PARAMS)
    timed.run(args.warmup)
    timed.synchronize()
    timed.reset_stats()
    timed.run(args.steps)
    timed.synchronize()
    ts = timed.stats()
    levels = [{"depth": d, "ms_per_launch": ms / args.steps, "cells_per_launch": cells // args.steps,
               "cells_per_s": cells / (ms / 1e3) if ms else None}
              for d, (ms, cells) in enumerate(timed.level_stats(DEPTH))]
    timed.close()
    per_launch_ms = ts["hist_ms"] / max(ts["hist_timed_launches"], 1)
    alg_bytes = ts["hist_cells"] + 12 * ts["hist_rows"]  # bins + row id + g/h per built row
    per_launch_bytes = alg_bytes / max(ts["hist_timed_launches"], 1)
    achieved = per_launch_bytes / (per_launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    # Whole tree: the histogram bytes above plus gradients (labels, predictions, weights in,
    # g/h pairs out: 32 B per row), the partitions (row id in, split feature's bin, row id
    # out: 9 B per routed row, rows counted on the device) and the prediction update (row
    # id, bin, prediction read and written: 21 B per row).
    part_rows = st["part_rows"] / args.steps
    tree_bytes = alg_bytes / args.steps + 32 * args.rows + 9 * part_rows + 21 * args.rows
    tree_achieved = tree_bytes / (ms_max / args.steps / 1e3) / 1e9

    # Plain paths. FP32 atomics in the same batched, graph-per-round trainer (the price of
    # exact fixed point alone), and FP32 atomics with one histogram launch per node and a
    # host round trip per level (the reference's MPS loop, mps_histogram.mm:62-80).
    def plain_rate(options, steps):
        t = mb.Trainer(backend, binned, y, w, n_estimators=steps + 2, options=options, **PARAMS)
        t.run(1)
        t.synchronize()
        backend.timer_begin()
        t.run(steps)
        ms = backend.timer_end()
        t.synchronize()
        t.close()
        return steps / (ms / 1e3)

    batched_fp32 = plain_rate(_lib.OPT_FLOAT_HIST, args.steps)
    per_node_fp32 = plain_rate(_lib.OPT_FLOAT_HIST | _lib.OPT_PER_NODE, max(2, args.steps // 4))

    # End to end through the C ABI: pinned host buffers in, model out, K trees; and the
    # same fit from ordinary (pageable) numpy arrays.
    e2e = e2e_pageable = None
    if rank == 0 or world > 1:
        e2e = run_e2e(mb, backend, binned, y, w, args.e2e_trees, pinned=True)
        # Fits from pageable memory vary with the host's state between runs (0.74-0.97 s
        # per 200-tree fit seen on the same build): the median of three fits.
        fits = sorted((run_e2e(mb, backend, binned, y, w, args.e2e_trees, pinned=False) for _ in range(3)),
                      key=lambda r: r["seconds"])
        e2e_pageable = dict(fits[1], fits_seconds=[round(r["seconds"], 4) for r in fits],
                            timing="median of three fits")
    trainer.close()
    secondary = run_secondary(mb, backend) if world == 1 and not args.no_secondary else None

    if rank != 0:
        return
    cpu = cpu_baseline(xf, y, w, args.cpu_rows, args.cpu_trees) if world == 1 and not args.no_cpu else None
    line = {
        "metric": METRIC, "value": value, "unit": "trees/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": dict(CONFIG, parallelism=f"replicas x{world}" if world > 1 else "single GPU",
                       binning_seconds=round(t_bin, 2), device_binning_seconds=round(t_dbin, 3),
                       device_binning_same_schema=dbin_equal,
                       launch_shape={k: tuning[k] for k in ("hist_threads", "hist_stages", "root_threads",
                                                             "items_per_sm", "blocked_levels", "scan_threads")},
                       autotune={"trials": tuning["trials"],
                                 "ms_per_round": round(tuning["ms_per_round"], 4),
                                 "built_in_ms_per_round": round(tuning["default_ms_per_round"], 4)}),
        "gpu_launches": int(st["kernel_launches"]),
        "e2e": e2e,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": HIST_TRAFFIC_PER_ALG_BYTE * per_launch_bytes,
                     "traffic_unit": "bytes per launch (ncu ratio at 4M rows x live algorithmic bytes)",
                     "traffic_source": HIST_TRAFFIC_PROFILE,
                     "peak_kind": peak_kind,
                     "kernel": "hist_build_direct_kernel (fixed point)",
                     "bytes_per_launch": per_launch_bytes, "ms_per_launch": per_launch_ms,
                     "cells_per_s": ts["hist_cells"] / (ts["hist_ms"] / 1e3), "levels": levels},
        "tree_roofline": {"bound": "hbm", "bytes_per_tree": tree_bytes, "ms_per_tree": ms_max / args.steps,
                          "achieved": tree_achieved, "peak": peak, "unit": "GB/s", "frac": tree_achieved / peak,
                          "roofline_trees_per_s": peak * 1e9 / tree_bytes,
                          "bytes": {"histogram": alg_bytes / args.steps, "gradients": 32 * args.rows,
                                    "partition": 9 * part_rows, "prediction_update": 21 * args.rows}},
        "plain_fp32_batched": {"value": batched_fp32, "unit": "trees/s",
                               "speedup_of_fixed_batched": value / world / batched_fp32,
                               "note": "FP32 shared atomics, FP64 node sums, same batched graph-per-round trainer"},
        "plain_fp32_per_node": {"value": per_node_fp32, "unit": "trees/s",
                                "speedup_of_fixed_batched": value / world / per_node_fp32,
                                "note": "FP32 atomics, one histogram launch per node, host round trip per level"},
        "e2e_pageable": e2e_pageable,
        "secondary": secondary,
        "cpu_baseline": cpu,
        "clocks": clocks_summary(samples),
    }
    print(json.dumps(line), flush=True)


def run_e2e(mb, backend, binned, y, w, trees, pinned=True):
    """One fit through mpsb_cuda_train_regressor: from page-locked host buffers (pinned;
    registered before the clock starts) or from ordinary numpy arrays (every cost inside
    the clock)."""
    import ctypes as C

    from mpsboost_gb300 import _lib

    lib = _lib.load()
    bins = np.ascontiguousarray(binned.bins)
    counts = np.ascontiguousarray(binned.bin_counts, np.uint32)
    yy = np.ascontiguousarray(y)
    ww = np.ascontiguousarray(w)
    registered = [bins, yy, ww] if pinned else []
    for a in registered:
        _lib.check(lib.mpsb_cuda_host_register(_lib.ptr(a), a.nbytes))
    try:
        p, keep = mb.make_params(n_estimators=trees, **PARAMS)
        t0 = time.perf_counter()
        ds = C.c_void_p()
        # The upload runs while the trainer checks labels and weights on the host.
        _lib.check(lib.mpsb_cuda_dataset_create_async(backend.handle, _lib.ptr(bins), 1, None, binned.rows,
                                                      binned.features, _lib.ptr(counts), C.byref(ds)))
        model = C.c_void_p()
        _lib.check(lib.mpsb_cuda_train_regressor(backend.handle, ds, _lib.ptr(yy), _lib.ptr(ww), yy.size,
                                                 C.byref(p), 0, C.byref(model)))
        nodes = 0
        for t in range(lib.mpsb_cuda_model_tree_count(model)):
            n = lib.mpsb_cuda_model_tree_node_count(model, t)
            out = np.empty(n, _lib.NODE_DTYPE)
            _lib.check(lib.mpsb_cuda_model_tree_nodes(model, t, _lib.ptr(out)))
            nodes += n
        dt = time.perf_counter() - t0
        lib.mpsb_cuda_model_destroy(model)
        lib.mpsb_cuda_dataset_destroy(ds)
        del keep
    finally:
        for a in registered:
            lib.mpsb_cuda_host_unregister(_lib.ptr(a))
    h2d = bins.nbytes + yy.nbytes + ww.nbytes + counts.nbytes
    d2h = nodes * _lib.NODE_DTYPE.itemsize  # the trees (training predictions stay on the device)
    return {"value": trees / dt, "unit": "trees/s", "h2d_bytes_per_step": h2d // trees,
            "d2h_bytes_per_step": d2h // trees, "seconds": dt,
            "host_memory": "page-locked (registered before timing)" if pinned else "pageable numpy arrays",
            "trees": trees,
            "note": "one fit of the configured model through mpsb_cuda_train_regressor: dataset upload "
                    "(asynchronous, beside the host's label and weight checks), training, tree readback. "
                    "It covers all rounds; later rounds split less evenly and build fewer cells (3.2e9 "
                    "per tree in rounds 181-200 against 3.9e9 in rounds 4-23, the rounds `value` times), "
                    "so its per-tree rate can exceed `value`"}


def run_secondary(mb, backend):
    """Bounded measurements of the other benchmark configurations on the same GPU.

    binary logistic 4M x 256 (10 % missing, depth 10, lr 0.1): trees/s over 8 graph-
    replayed rounds, CUDA events on the backend stream, device-binned data resident.
    one-vs-rest K = 10, 2M x 64, depth 6: per round from one-shot fits through the public
    API (medians of three fits of 20 and of 4 rounds; the difference removes setup), 10
    trees per round.
    random forest 1M x 100, 256 trees, depth 12, sqrt features, Poisson(1) rows: one
    host-timed fit of the whole forest through the public API (sample expansion, upload,
    training, model readback) after a 16-tree warm-up.
    wide bins: the regression workload's generator at 4M rows with max_bins 1024 (u16
    bins, 1024 histogram slots per feature), device-binned; trees/s over 8 graph-replayed
    rounds, CUDA events."""
    out = {}
    xf, y, w = make_data(4_000_000)
    dset = mb.quantize_device(backend, xf.T, 1024)
    del xf
    params = dict(PARAMS, max_bins=1024)
    t = mb.Trainer(backend, dset, y, w, n_estimators=12, **params)
    t.run(3)
    t.synchronize()
    backend.timer_begin()
    t.run(8)
    ms = backend.timer_end()
    t.synchronize()
    t.close()
    dset.close()
    out["regression_1024bins_4Mx128_d8"] = {"value": 8 / (ms / 1e3), "unit": "trees/s", "ms_per_tree": ms / 8,
                                            "rounds": 8, "timing": "CUDA events, graph per round"}
    del y, w

    x, y = make_logistic_data()
    dset = mb.quantize_device(backend, x, 255)
    del x
    params = dict(max_depth=10, learning_rate=0.1, objective="binary_logistic", min_samples_leaf=20,
                  min_child_weight=1.0, reg_lambda=1.0, max_bins=255)
    t = mb.Trainer(backend, dset, y, None, n_estimators=12, **params)
    t.run(3)
    t.synchronize()
    backend.timer_begin()
    t.run(8)
    ms = backend.timer_end()
    t.synchronize()
    t.close()
    dset.close()
    out["logistic_4Mx256_d10"] = {"value": 8 / (ms / 1e3), "unit": "trees/s", "ms_per_tree": ms / 8,
                                  "rounds": 8, "timing": "CUDA events, graph per round"}
    del y

    x, labels = make_ovr_data()
    dset = mb.quantize_device(backend, x, 255)
    del x
    params = dict(max_depth=6, learning_rate=0.1, min_samples_leaf=20, min_child_weight=1.0, reg_lambda=1.0)
    mb.train_ovr(backend, dset, labels, 10, n_estimators=2, **params)  # warm
    times = {4: [], 20: []}
    for _ in range(3):
        for rounds in (4, 20):
            backend.synchronize()
            t0 = time.perf_counter()
            mb.train_ovr(backend, dset, labels, 10, n_estimators=rounds, **params)
            times[rounds].append(time.perf_counter() - t0)
    dset.close()
    t4, t20 = statistics.median(times[4]), statistics.median(times[20])
    per_round = (t20 - t4) / 16
    out["ovr_k10_2Mx64_d6"] = {"value": 10 / per_round, "unit": "trees/s", "ms_per_round": per_round * 1e3,
                               "fit_seconds_20_rounds": t20,
                               "timing": "host, (median t(20) - median t(4)) / 16 over three fits each"}
    del labels

    x, y, counts, subsets = make_forest_data()
    binned = mb.quantize_dense(x, 255)
    del x
    params = dict(max_depth=12, min_samples_leaf=20, max_bins=255)
    mb.train_forest(backend, binned, y, row_counts=counts[:16], feature_subsets=subsets[:16], **params)
    backend.synchronize()
    t0 = time.perf_counter()
    models = mb.train_forest(backend, binned, y, row_counts=counts, feature_subsets=subsets, **params)
    dt = time.perf_counter() - t0
    out["forest_256_1Mx100_d12"] = {"value": len(models) / dt, "unit": "trees/s", "seconds_per_forest": dt,
                                    "timing": "host, whole forest through the public API"}
    return out


def run_forest(args, rank, world):
    """Random-forest regression: 1,000,000 rows x 100 N(0,1) features, Friedman-1 target on
    x0..x4 + N(0,1); 256 trees, per-tree Poisson(1) row weights, 10 = sqrt(100) features per
    tree, depth 12, min_samples_leaf 20; every tree of a batch built in the same launches.
    A step is one forest of ``--forest-trees`` trees."""
    import mpsboost_gb300 as mb

    trees = args.forest_trees
    x, y, counts, subsets = make_forest_data(trees=trees)
    binned = mb.quantize_dense(x, 255)
    backend = mb.CudaBackend(int(os.environ.get("LOCAL_RANK", "0")))
    params = dict(max_depth=12, min_samples_leaf=20, max_bins=255)
    for _ in range(args.warmup):
        mb.train_forest(backend, binned, y, row_counts=counts[: min(trees, 16)],
                        feature_subsets=subsets[: min(trees, 16)], **params)
    times, nodes = [], 0
    for _ in range(args.steps):
        barrier(world)
        t0 = time.perf_counter()
        models = mb.train_forest(backend, binned, y, row_counts=counts, feature_subsets=subsets, **params)
        times.append(time.perf_counter() - t0)
        nodes = sum(len(m.trees[0]) for m in models)
    dt = reduce_max(statistics.median(times), world)
    if rank == 0:
        print(json.dumps({"metric": "forest trees/s @1Mx100 d12 sqrt-features Poisson(1)",
                          "value": world * trees / dt, "unit": "trees/s", "n_gpus": world,
                          "steps": args.steps, "warmup": args.warmup, "seconds_per_forest": dt,
                          "trees": trees, "nodes": nodes, "dtype": "int64", "data": "synthetic",
                          "note": "host-timed fit of the whole forest (sample expansion, upload, "
                                  "training, model readback), binned data resident"}), flush=True)


def run_logistic(args, rank, world):
    """Binary logistic configuration: 4M x 256 (10 % missing cells), depth 10, lr 0.1,
    device-binned to 255 bins; K graph-replayed rounds after W warm-up rounds, CUDA events
    (rows from --rows when given below the default)."""
    import mpsboost_gb300 as mb

    rows = min(args.rows, 4_000_000)
    x, y = make_logistic_data(rows)
    backend = mb.CudaBackend(int(os.environ.get("LOCAL_RANK", "0")))
    dset = mb.quantize_device(backend, x, 255)
    del x
    params = dict(max_depth=10, learning_rate=0.1, objective="binary_logistic", min_samples_leaf=20,
                  min_child_weight=1.0, reg_lambda=1.0, max_bins=255)
    t = mb.Trainer(backend, dset, y, None, n_estimators=args.warmup + args.steps + 1, **params)
    t.run(args.warmup)
    t.synchronize()
    barrier(world)
    backend.timer_begin()
    t.run(args.steps)
    ms = reduce_max(backend.timer_end(), world)
    t.synchronize()
    st = t.stats()
    t.close()
    if rank == 0:
        print(json.dumps({"metric": "trees/s @4Mx256 logistic d10", "value": world * args.steps / (ms / 1e3),
                          "unit": "trees/s", "rows": rows, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_tree": ms / args.steps, "gpu_launches": int(st["kernel_launches"]),
                          "dtype": "int64", "data": "synthetic"}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-rows", type=int, default=500_000)
    ap.add_argument("--cpu-trees", type=int, default=5,
                    help="trees of the CPU baseline sample (about 10 s of single-core training)")
    ap.add_argument("--ref-rows", type=int, default=500_000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--e2e-trees", type=int, default=TREES,
                    help="trees of the end-to-end fit (default: the configuration's 200)")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the bounded logistic / one-vs-rest / forest measurements")
    ap.add_argument("--rows", type=int, default=ROWS,
                    help="rows of the synthetic workload (profiling runs use fewer)")
    ap.add_argument("--workload", choices=["regression", "forest", "logistic"], default="regression",
                    help="forest: the 256-tree random-forest configuration instead of the default; "
                         "logistic: the binary-logistic configuration's training rounds")
    ap.add_argument("--forest-trees", type=int, default=256)
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the built-in launch shape (profiling runs)")
    ap.add_argument("--only-train", action="store_true",
                    help="time the training rounds only (for launch lists and ncu captures)")
    ap.add_argument("--max-bins", type=int, default=BINS,
                    help="with --only-train: bins per feature (above 256: u16 bins, the wide kernels)")
    args = ap.parse_args()
    if args.max_bins != BINS and not args.only_train:
        ap.error("--max-bins applies to --only-train runs")
    if args.warmup < 3:
        args.warmup = 3
    rank, world = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "forest":
        run_forest(args, rank, world)
    elif args.workload == "logistic":
        run_logistic(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
