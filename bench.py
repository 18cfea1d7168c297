"""Benchmark: batched NUFFT forward + adjoint throughput (Msamples/s).

Default workload (the headline): configuration 2, 2-D 256^2 image x 8 coils,
golden-angle radial 402 spokes x 512 samples, oversampled grid 512^2, nspread 6.
``--workload c1..c5`` measures the other configurations the same way:
  c1  2-D 128^2, 1 coil, uniform radial 128 x 256
  c3  64 frames x 12 coils of 192^2, ragged golden-angle spokes U{5..34} x 384
  c4  3-D 128^3 x 8 coils, 20,000 centre-out spokes x 128 (256^3 grid)
  c5  2-D 256^2 x 16 coils, variable-density spiral 24 x 2048, perturbed coordinates

One step = type-2 (forward) + type-1 (adjoint) over every instance (group x coil),
replayed from one CUDA graph; value = (samples x coils) / step time.  Also reported:
  plain        the per-instance path: single-coil plans, eager launches, instance by instance
  e2e          the same step through the C ABI with pinned host buffers, H2D and D2H inside
               the timed region (gbn_type2_host + gbn_type1_host)
  roofline     dominant gridding kernel: algorithmic bytes / its CUDA-event time vs the
               measured HBM copy bandwidth, with the FP32 rate beside it; "binding" gives
               the fraction of the resource that bounds the kernel (HBM, FP32 or shared memory)
  tiling       tiles, threads and coils per block, chosen by the autotuner on the
               workload's trajectory before the timed region (--tune off: library defaults)
  cpu_baseline the FP64 C restatement of mripy's CPU NUFFT on the host cores
  accuracy     relative L2 error vs the FP64 NUDFT on a subset
  solver       c2: 20 CG-SENSE iterations; c4: Pipe-Menon dcf + 30 IST iterations with a
               level-4 Haar L1 prox (each iteration one CUDA graph)
  autograd     c5: loss ||A(x; k) - y||^2 and its gradients with respect to image and trajectory
  --part espirit / haar (c2, c4): ESPIRiT coil maps and the Haar transform / wavelet prox on
               the workload's coil data, beside their FP64 host restatements

--impl reference times mripy's CPU NUFFT algorithm (the oracle port; mripy itself is
Python + numba and is not installed on the GPU host) on the same workload.
Under torchrun (N > 1) every rank runs its own replica (weak scaling, no collective in
the data path); rank 0 prints the line with the max step time over ranks.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched NUFFT fwd+adj Msamples/s vs per-instance plain at ≤1e-4 rel err"
UNIT = "Msamples/s"
L2_BYTES = 129 * 2 ** 20
# plan info's spread_variant -> the spread kernel that ran
SPREAD_KERNELS = {3: "k_spread_mma: tensor cores (+ compensated instance for dense tiles)",
                  2: "k_spread3d_cube: FP32 register cubes", 1: "k_spread3d_reg: warp rows",
                  0: "register tiles (2-D) or shared-memory tiles"}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value):
    """Max of a host float over all ranks (identity without torch.distributed)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_units(units_per_replica, world):
    """Weak scaling: every rank processes its own replica of the workload."""
    return units_per_replica * world


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _sm_max_mhz():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["sm_max_mhz"])
    except Exception:
        return 2070.0


def tf32_peak_tflops():
    """TF32 tensor rate: half the measured cuBLAS BF16 burst rate (MEASURED_PEAKS.json), else
    half the fallback 1.9 PFLOP/s."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["bf16_tflops"]) / 2
    except Exception:
        return 1900.0 / 2


def fp32_peak_tflops():
    """Nominal FP32 CUDA-core peak: 152 SMs x 128 FMA lanes x 2 flop x max SM clock."""
    return 152 * 128 * 2 * _sm_max_mhz() * 1e6 / 1e12


def smem_peak_tbs():
    """Nominal shared-memory read bandwidth: 152 SMs x 128 B/clk x max SM clock."""
    return 152 * 128 * _sm_max_mhz() * 1e6 / 1e12


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 20 ms; only samples whose
    nvidia-smi timestamp falls inside the marked timed window are summarised."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.5)  # let the sampler come up before the timed window opens
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def mark_start(self):
        import datetime
        self.t0 = datetime.datetime.now()

    def mark_end(self):
        import datetime
        self.t1 = datetime.datetime.now()

    def stop(self):
        import datetime
        if self.proc is None:
            return None
        time.sleep(0.1)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        pad = datetime.timedelta(milliseconds=25)
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f")
                mhz = float(parts[2])
                smax = max(smax, float(parts[3]))
            except ValueError:
                continue
            if self.t0 is not None and not (self.t0 - pad <= ts <= self.t1 + pad):
                continue
            sm.append(mhz)
            for n, v in zip(names, parts[6:10]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": smax or None, "reasons": [],
                    "samples": 0, "note": "timed window shorter than the 20 ms sampling period"}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------------------ workloads

class Workload:
    def __init__(self, name, description, dim, shape, coords, imgs, n_coil, offsets=None, eps=5e-6,
                 max_nspread=None, sens=None, base_image=None):
        self.name, self.description, self.dim, self.shape = name, description, dim, tuple(shape)
        self.coords = [np.ascontiguousarray(c, dtype=np.float64) for c in coords]   # radians
        self.imgs = imgs                      # (n_traj, *shape, n_coil) complex64
        self.n_coil = n_coil
        self.M = len(self.coords[0])
        self.offsets = list(offsets) if offsets is not None else [0, self.M]
        self.n_traj = len(self.offsets) - 1
        self.eps, self.max_nspread = eps, max_nspread
        self.sens, self.base_image = sens, base_image


def make_workload(name):
    from mripy_gb300 import synth
    two_pi = 2 * np.pi
    if name == "c1":
        cfg = synth.config1()
        return Workload("c1", "2-D 128^2, 1 coil, uniform radial 128x256, 256^2 grid, nspread 6", 2, (128, 128),
                        [two_pi * k for k in cfg["k"]], cfg["image"][None, ..., None], 1)
    if name == "c2":
        cfg = synth.config2()
        imgs = (cfg["image"][..., None] * cfg["sens"]).astype(np.complex64)[None]
        return Workload("c2", "2-D 8-coil golden-angle radial 402x512 samples, 256^2 image, 512^2 grid, "
                        "nspread 6 (eps 5e-6)", 2, (256, 256), [two_pi * k for k in cfg["k"]], imgs, 8,
                        sens=cfg["sens"], base_image=cfg["image"])
    if name == "c3":
        cfg = synth.config3()
        return Workload("c3", "64 frames x 12 coils of 192^2, ragged golden-angle spokes U{5..34} x 384, "
                        "384^2 grid, nspread 6", 2, (192, 192), [two_pi * k for k in cfg["k"]], cfg["image"], 12,
                        offsets=cfg["offsets"])
    if name == "c4":
        cfg = synth.config4()
        imgs = (cfg["image"][..., None] * cfg["sens"]).astype(np.complex64)[None]
        return Workload("c4", "3-D 128^3 x 8 coils, 20000 centre-out spokes x 128 (Fibonacci sphere), 256^3 grid, "
                        "nspread 6", 3, (128, 128, 128), [two_pi * k for k in cfg["k"]], imgs, 8, max_nspread=6,
                        sens=cfg["sens"], base_image=cfg["image"])
    if name == "c5":
        cfg = synth.config5()
        return Workload("c5", "2-D 256^2 x 16 coils, variable-density spiral 24x2048, perturbed coordinates, "
                        "512^2 grid, nspread 6", 2, (256, 256), [two_pi * k for k in cfg["k_perturbed"]],
                        cfg["image"][None], 16)
    raise ValueError("unknown workload " + name)


def line_config(wl, nf, nspread, world=1):
    """The workload keys of the JSON line, identical in the GPU arm and the reference arm."""
    return {"workload": wl.description, "samples": wl.M, "coils": wl.n_coil, "groups": wl.n_traj,
            "image": list(wl.shape), "grid": [int(v) for v in nf], "nspread": int(nspread),
            "step": "type-2 + type-1 over all instances (group x coil)",
            "l2": "GPU arm: flushed between timed steps (write of %d MiB)" % (2 * L2_BYTES // 2 ** 20),
            "parallelism": "replicas, one per rank" if world > 1 else "single GPU"}


def algorithmic_bytes(M, n_coil, dim, grid_cells, n_inst):
    """Per direction: samples (complex64, every coil) + packed coordinates read once per
    shared trajectory (4 B per dim) + the oversampled grid of every instance (complex64)."""
    return 8 * M * n_coil + 4 * dim * M + 8 * grid_cells * n_inst


def stencil_footprint(coords, offsets, nf, ns):
    """Grid cells inside at least one sample's stencil, summed over trajectory groups: the
    cells an interp must read at least once.  A sample at x (radians) has its first tap at
    ((1 + floor((x mod 2 pi) / h)) - ns) mod nf, h = 2 pi / nf, and W = 2 ns taps per axis,
    as the prep kernel places it."""
    W = 2 * ns
    total = 0
    for g in range(len(offsets) - 1):
        a, b = int(offsets[g]), int(offsets[g + 1])
        if b <= a:
            continue
        idx = []
        for d, x in enumerate(coords):
            h = 2 * np.pi / nf[d]
            m = 1 + np.floor(np.mod(np.asarray(x[a:b], dtype=np.float64), 2 * np.pi) / h).astype(np.int64)
            idx.append((m - ns) % nf[d])
        occ = np.zeros(tuple(nf), dtype=bool)
        occ[tuple(idx)] = True
        for d in range(len(nf)):
            cov = occ.copy()
            for sft in range(1, W):
                cov |= np.roll(occ, sft, axis=d)
            occ = cov
        total += int(np.count_nonzero(occ))
    return total


def flops(M, n_coil, W, dim):
    T = W ** dim
    return 4 * T * M * n_coil + T * M


def event_time(torch, fn, reps, stream, flush=None):
    """CUDA-event time of each call of fn on ``stream``; the L2 flush between calls is
    outside the event pairs.  One host synchronisation at the end."""
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    for i in range(reps):
        if flush is not None:
            flush()
        starts[i].record(stream)
        fn()
        ends[i].record(stream)
    ends[-1].synchronize()
    ts = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    return float(np.median(ts)), ts


def run_gpu(args, wl):
    import torch
    from mripy_gb300 import _native as N
    from mripy_gb300.plan import NufftPlan

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    coords = [torch.from_numpy(c).to(dev) for c in wl.coords]
    img = torch.from_numpy(np.ascontiguousarray(wl.imgs)).to(dev)           # (n_traj, *shape, n_coil)
    M, n_coil, n_inst = wl.M, wl.n_coil, wl.n_traj * wl.n_coil
    samples = torch.empty((M, n_coil), dtype=torch.complex64, device=dev)
    out_img = torch.empty_like(img)
    tuning, tune_s = None, None
    if args.tune == "auto":
        # the autotuner times candidate tilings on this trajectory (outside the timed region)
        from mripy_gb300.tune import autotune
        t0 = time.perf_counter()
        tuning = autotune(wl.dim, wl.shape, coords, n_coil=n_coil, n_traj=wl.n_traj, traj_offsets=wl.offsets,
                          eps=wl.eps, cache_file=args.tune_cache)
        tune_s = time.perf_counter() - t0
    plan = NufftPlan(wl.dim, wl.shape, n_coil=n_coil, n_traj=wl.n_traj, eps=wl.eps, max_nspread=wl.max_nspread,
                     tuning=tuning)
    plan.set_points(coords, traj_offsets=wl.offsets)
    info = plan.info()
    stream = torch.cuda.current_stream()
    flush_buf = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    def flush():
        flush_buf.fill_(1.0)

    # --- batched step captured in one CUDA graph (type-2 then type-1 on fixed buffers)
    def step_eager():
        plan.type2(img, out=samples)
        plan.type1(samples, out=out_img)

    step_eager()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        step_eager()
    stream.wait_stream(side)
    torch.cuda.synchronize()
    with torch.cuda.graph(g):
        step_eager()
    torch.cuda.synchronize()

    for _ in range(args.warmup):
        flush()
        g.replay()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    torch.cuda.synchronize()
    if sampler:
        sampler.mark_start()
    t_wall = time.perf_counter()
    _, step_ms = event_time(torch, g.replay, args.steps, stream, flush)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    if sampler:
        sampler.mark_end()
    clocks = sampler.stop() if sampler else None
    mean_ms = max_over_ranks(float(np.mean(step_ms)))
    value = replica_units(M * n_coil, world) / (mean_ms * 1e-3) / 1e6

    result = {"metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
              "warmup": args.warmup, "ms_per_step": round(mean_ms, 4), "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None, "dtype": "c64",
              "data": "synthetic (seeded phantoms/random images x coil maps, %s)" % wl.description,
              "config": line_config(wl, info["nf"], info["nspread"], world),
              "tiling": {"spread_tile": list(info["spread_tile"]), "interp_tile": list(info["interp_tile"]),
                         "spread_coils_per_block": info["coil_group"],
                         "interp_coils_per_block": info["interp_coil_group"],
                         "spread_threads": info["threads"], "interp_threads": info["interp_threads"],
                         "max_subproblem": info["max_subproblem"],
                         "spread_kernel": SPREAD_KERNELS.get(info["spread_variant"], "shared-memory tiles"),
                         "interp_kernel": ("k_interp3d_mma: tensor cores on the spread's tiles (8 coils per block; "
                                           "interp_tile and interp_* above do not apply)"
                                           if info["interp_variant"] == 2 else "interp bins (interp_tile)"),
                         "chosen_by": "autotuner (%.1f s, untimed)" % tune_s if tuning is not None
                         else "library defaults"},
              "wall_s_timed": round(t_wall, 3)}
    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return None

    # --- per-kernel timing (stages alone, same stream, L2 flushed)
    grid = plan.grid()
    plan.pad_deapod(img, grid)
    plan.fft(grid, N.GBN_FFT_FORWARD)
    grid_copy = grid.clone()
    reps = 20 if wl.dim == 2 else 5
    t_interp, _ = event_time(torch, lambda: plan.interp(grid_copy, out=samples), reps, stream, flush)
    t_spread, _ = event_time(torch, lambda: plan.spread(samples, grid), reps, stream, flush)
    t_pad, _ = event_time(torch, lambda: plan.pad_deapod(img, grid), reps, stream, flush)
    # the step's transforms: pruned to the image band where the plan says so (fft_variant 2)
    t_fft, _ = event_time(torch, lambda: plan.fft_band(grid, N.GBN_FFT_FORWARD, N.GBN_BAND_INPUT), reps, stream, flush)
    t_fft_inv, _ = event_time(torch, lambda: plan.fft_band(grid, N.GBN_FFT_INVERSE, N.GBN_BAND_OUTPUT), reps, stream,
                              flush)
    t_fft_full, _ = event_time(torch, lambda: plan.fft(grid, N.GBN_FFT_FORWARD), reps, stream, flush)
    t_crop, _ = event_time(torch, lambda: plan.crop_deapod(grid, out_img), reps, stream, flush)
    del grid_copy
    G = info["grid_cells"]
    bytes_dir = algorithmic_bytes(M, n_coil, wl.dim, G, n_inst)
    fl = flops(M, n_coil, 2 * info["nspread"], wl.dim)
    hbm, peak_kind = peaks()
    dominant = "spread" if t_spread >= t_interp else "interp"
    t_dom = max(t_spread, t_interp)
    achieved = bytes_dir / (t_dom * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "ncu_traffic_%s.txt" % wl.name)
    if os.path.exists(tpath):
        for ln in open(tpath):
            if ln.startswith(dominant + "_dram_bytes_per_launch:"):
                traffic = int(ln.split(":")[1])
    result["roofline"] = {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1),
                          "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 4), "traffic": traffic,
                          "peak_source": ("of measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                                          else "of fallback 6.8 TB/s"),
                          "algorithmic_bytes_per_launch": bytes_dir,
                          "fp32_tflops_achieved": round(fl / (t_dom * 1e-3) / 1e12, 2)}
    # interp bytes counting only the grid cells some stencil reaches (the spread writes the
    # whole grid, so its bytes stay on the full grid)
    fp_cells = stencil_footprint(wl.coords, wl.offsets, info["nf"], info["nspread"])
    interp_bytes_fp = 8 * M * n_coil + 4 * wl.dim * M + 8 * fp_cells * n_coil
    result["roofline"]["interp_footprint"] = {
        "cells_touched": fp_cells, "grid_cells": G * wl.n_traj, "frac_of_grid": round(fp_cells / (G * wl.n_traj), 4),
        "interp_bytes_footprint": interp_bytes_fp, "interp_bytes_full_grid": bytes_dir,
        "interp_gbs_footprint": round(interp_bytes_fp / (t_interp * 1e-3) / 1e9, 1),
        "interp_gbs_full_grid": round(bytes_dir / (t_interp * 1e-3) / 1e9, 1)}
    # the stencil kernels are bound by arithmetic (spread) or shared-memory reads (interp)
    # rather than HBM: the binding resource is the largest of the three demand/peak times
    fp32_peak = fp32_peak_tflops()
    smem_peak = smem_peak_tbs()
    demand = {"hbm": bytes_dir / (hbm * 1e9), "fp32": fl / (fp32_peak * 1e12)}
    if dominant == "interp":
        T = (2 * info["nspread"]) ** wl.dim
        icg = info["interp_coil_group"]
        smem_bytes = 8 * T * M * icg * ((n_coil + icg - 1) // icg)   # every tap of every coil lane read once
        demand["smem"] = smem_bytes / (smem_peak * 1e12)
    bind = max(demand, key=demand.get)
    result["roofline"]["binding"] = {
        "resource": bind, "frac": round(demand[bind] / (t_dom * 1e-3), 4),
        "fracs": {k: round(v / (t_dom * 1e-3), 4) for k, v in demand.items()},
        "peaks": {"hbm_gbs": hbm, "fp32_tflops": round(fp32_peak, 1), "smem_tbs": round(smem_peak, 1)},
        "peak_note": "FP32 and shared-memory peaks are nominal (152 SMs x 128 FMA lanes, x 128 B/clk) at the "
                     "measured max SM clock"}
    if info.get("interp_variant") == 2:
        # the tensor-core interp: per (sample, tile) pair 3 TF32 MMAs' worth of M = 128
        # samples x N = 64 over K = 128 (y, z) cells, as the spread
        mma_flop_i = info["spread_entries"] * 3 * 2 * 128 * 64
        result["roofline"]["interp_tensor"] = {
            "kernel": "k_interp3d_mma", "mma_tflop_per_launch": round(mma_flop_i / 1e12, 3),
            "achieved_tflops": round(mma_flop_i / (t_interp * 1e-3) / 1e12, 1),
            "peak_tflops": round(tf32_peak_tflops(), 1),
            "frac": round(mma_flop_i / (t_interp * 1e-3) / 1e12 / tf32_peak_tflops(), 4),
            "peak_source": "of measured (MEASURED_PEAKS.json bf16_tflops / 2: TF32 at half the BF16 rate)"}
    if info.get("spread_variant") == 3:
        # the tensor-core spread: 3 TF32 MMAs (hi*hi, hi*lo, lo*hi) of M = 128 cells x N = 64
        # (4 x-planes x 8 coils x re/im) per (sample, tile) pair; TF32 runs at half the BF16
        # rate, so the reference is the measured cuBLAS BF16 burst / 2
        mma_flop = info["spread_entries"] * 3 * 2 * 128 * 64
        tf32_peak = tf32_peak_tflops()
        result["roofline"]["spread_tensor"] = {
            "kernel": "k_spread_mma<3, ...>", "mma_tflop_per_launch": round(mma_flop / 1e12, 3),
            "achieved_tflops": round(mma_flop / (t_spread * 1e-3) / 1e12, 1), "peak_tflops": round(tf32_peak, 1),
            "frac": round(mma_flop / (t_spread * 1e-3) / 1e12 / tf32_peak, 4),
            "peak_source": "of measured (MEASURED_PEAKS.json bf16_tflops / 2: TF32 at half the BF16 rate)",
            "stencil_fp32_tflops": round(fl / (t_spread * 1e-3) / 1e12, 2),
            "stencil_fp32_frac": round(fl / (t_spread * 1e-3) / 1e12 / fp32_peak, 4)}
    result["kernels_ms"] = {"interp": round(t_interp, 4), "spread": round(t_spread, 4), "pad_deapod": round(t_pad, 4),
                            "fft": round(t_fft, 4), "fft_inverse": round(t_fft_inv, 4),
                            "fft_full_transform": round(t_fft_full, 4), "crop_deapod": round(t_crop, 4),
                            "fft_pruned_to_band": info["fft_variant"] == 2}
    # this library's kernels per step (cuFFT and memsets not counted): pad, interp, crop and
    # what the spread launched in the eager step before capture (split-tile zeroing unless the
    # grid is cleared by a memset; the 3-D compensated instance for dense tiles)
    per_step = 2 + (1 if info["interp_subproblems"] else 0) + plan.info()["spread_kernels"]
    result["gpu_launches"] = per_step * args.steps

    # --- plain per-instance path: single-coil plan per group, eager, instance by instance
    plans = []
    for gi in range(wl.n_traj):
        a, b = wl.offsets[gi], wl.offsets[gi + 1]
        p1 = NufftPlan(wl.dim, wl.shape, n_coil=1, eps=wl.eps, max_nspread=wl.max_nspread)
        p1.set_points([c[a:b] for c in coords])
        plans.append((p1, torch.empty((b - a, 1), dtype=torch.complex64, device=dev),
                      [img[gi, ..., c:c + 1].contiguous()[None] for c in range(n_coil)]))
    o1 = torch.empty((1,) + wl.shape + (1,), dtype=torch.complex64, device=dev)

    def plain_step():
        for p1, s1, coil_imgs in plans:
            for ci in coil_imgs:
                p1.type2(ci, out=s1)
                p1.type1(s1, out=o1)

    for _ in range(2):
        plain_step()
    t_plain, _ = event_time(torch, plain_step, min(20, max(3, args.steps // 10)), stream, flush)
    result["plain"] = {"value": round(M * n_coil / (t_plain * 1e-3) / 1e6, 2), "unit": UNIT,
                       "ms_per_step": round(t_plain, 4), "speedup_batched_vs_plain": round(t_plain / mean_ms, 2)}
    for p1, _, _ in plans:
        p1.close()
    del plans

    # --- accuracy vs the exact FP64 sums (NUDFT), every coil of every group
    plan.type2(img, out=samples)
    plan.type1(samples, out=out_img)
    torch.cuda.synchronize()
    result["accuracy"] = accuracy_vs_nudft(wl, samples.cpu().numpy(), out_img.cpu().numpy())

    # --- end to end through the C ABI with pinned host buffers
    h_img = torch.from_numpy(np.ascontiguousarray(wl.imgs)).pin_memory()
    h_k = torch.empty((M, n_coil), dtype=torch.complex64).pin_memory()
    h_out = torch.empty_like(h_img).pin_memory()
    lib = N.lib()
    sp = ctypes.c_void_p(stream.cuda_stream)

    def e2e_step():
        N.check(lib.gbn_type2_host(plan._h, ctypes.c_void_p(h_img.data_ptr()), ctypes.c_void_p(h_k.data_ptr()), sp))
        N.check(lib.gbn_type1_host(plan._h, ctypes.c_void_p(h_k.data_ptr()), ctypes.c_void_p(h_out.data_ptr()), sp))

    for _ in range(2):
        e2e_step()
    ts = []
    for _ in range(min(50 if wl.dim == 2 else 5, max(3, args.steps))):
        flush()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        ts.append(time.perf_counter() - t0)
    t_e2e = float(np.median(ts))  # host wall clock: the median discards scheduler hiccups
    img_bytes = wl.imgs.nbytes
    k_bytes = M * n_coil * 8
    result["e2e"] = {"value": round(M * n_coil / t_e2e / 1e6, 2), "unit": UNIT,
                     "h2d_bytes_per_step": img_bytes + k_bytes, "d2h_bytes_per_step": k_bytes + img_bytes,
                     "ms_per_step": round(t_e2e * 1e3, 3),
                     "path": "gbn_type2_host + gbn_type1_host (host pinned buffers, includes H2D and D2H)"}

    # --- solver: 20 CG-SENSE iterations (c2) / 30 IST iterations with a Haar-wavelet L1 prox
    # (c4), every iteration one CUDA graph of the normal operator and the solver kernels
    if wl.name == "c2":
        result["solver"] = cg_sense_time(torch, wl, coords)
    if wl.name == "c4":
        result["solver"] = ist_time(torch, wl, tuning)
    if wl.name == "c5":
        result["autograd"] = autograd_time(torch, wl, tuning)

    # --- CPU baseline: FP64 port of mripy's CPU NUFFT on the host cores (bounded sample)
    result["cpu_baseline"] = cpu_baseline_subprocess(wl)
    if clocks:
        result["clocks"] = clocks
    if world > 1:
        torch.distributed.barrier()
    return result


def accuracy_vs_nudft(wl, cf, of, seed=1):
    """Relative L2 error of the step's type-2 samples and type-1 images against the exact
    FP64 sums, over every coil of every group: per group a random sample subset for type-2
    and a random pixel box (the outer product of per-axis index lists) for type-1, about
    4096 of each in all (at least 512 per group in 3-D)."""
    import oracle as O
    rng = np.random.default_rng(seed)
    d, G = wl.dim, wl.n_traj
    n_s = max(64, 4096 // G) if d == 2 else 512
    side = max(8, int(round((4096 // G) ** (1.0 / d)))) if d == 2 else 8
    num_f = den_f = num_a = den_a = 0.0
    worst = 0.0
    for g in range(G):
        a, b = wl.offsets[g], wl.offsets[g + 1]
        if b <= a:
            continue
        xs = tuple(c[a:b] for c in wl.coords)
        sub = np.sort(rng.choice(b - a, min(n_s, b - a), replace=False))
        ex = O.nudft_type2_at(xs, wl.imgs[g].astype(np.complex128), wl.shape, sub)        # (n, coils)
        got = cf[a + sub].astype(np.complex128)
        num_f += np.sum(np.abs(got - ex) ** 2)
        den_f += np.sum(np.abs(ex) ** 2)
        pa = [np.sort(rng.choice(m, min(side, m), replace=False)) for m in wl.shape]
        exa = O.nudft_type1_box(xs, cf[a:b].astype(np.complex128), wl.shape, pa)        # (*box, coils)
        ga = of[g][np.ix_(*pa)].astype(np.complex128)
        num_a += np.sum(np.abs(ga - exa) ** 2)
        den_a += np.sum(np.abs(exa) ** 2)
        per_coil = np.linalg.norm((got - ex).reshape(-1, wl.n_coil), axis=0) / \
            np.linalg.norm(ex.reshape(-1, wl.n_coil), axis=0)
        worst = max(worst, float(per_coil.max()))
    return {"fwd_rel_l2_vs_nudft": float("%.3e" % np.sqrt(num_f / den_f)),
            "adj_rel_l2_vs_nudft": float("%.3e" % np.sqrt(num_a / den_a)),
            "fwd_worst_coil_group": float("%.3e" % worst), "target": 1e-4,
            "subset": "every coil of all %d group(s): %d samples and a %s pixel box per group" % (
                G, n_s, "x".join([str(side)] * d))}


def cg_sense_time(torch, wl, coords):
    from mripy_gb300 import operators as ops
    from mripy_gb300 import solvers
    nft = ops.NUFFT2d(wl.shape)
    nft.set_ktraj(coords[0], coords[1])
    A = ops.joint2operators(ops.espirit(wl.sens), nft)
    x = torch.from_numpy(wl.base_image).cuda()[..., None]
    y = A.forward(x)
    rng = np.random.default_rng(2)
    sigma = float(torch.linalg.vector_norm(y)) / np.sqrt(y.numel()) * 10 ** (-30 / 20)
    noise = torch.from_numpy((rng.standard_normal(tuple(y.shape)) + 1j * rng.standard_normal(tuple(y.shape)))
                             .astype(np.complex64) * sigma / np.sqrt(2)).cuda()
    y = y + noise
    solvers.cg_sense(A, y, n_iter=20)             # warm-up (plans, graph)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xr, norms = solvers.cg_sense(A, y, n_iter=20)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    # relative error against the phantom after a least-squares scale
    xt = x.reshape(-1)
    xh = xr.reshape(-1)
    a = torch.vdot(xh, xt) / torch.vdot(xh, xh)
    err = float(torch.linalg.vector_norm(a * xh - xt) / torch.linalg.vector_norm(xt))
    return {"cg_sense_iterations": 20, "ms_total": round(dt * 1e3, 2),
            "ms_per_iteration": round(dt * 1e3 / 20, 3), "residual_reduction": float("%.3e" % float(norms[-1] / norms[0])),
            "rel_error_vs_phantom": round(err, 4), "noise": "complex Gaussian, 30 dB SNR"}


def ist_time(torch, wl, tuning):
    """3-D UTE IST with wavelet L1: dcf by Pipe-Menon iteration (the trajectory comes without
    one), SENSE operator joint2operators(espirit, NUFFT3d), data scaled by optscaling, and
    IST_wrap with DWTnd('haar', level 4), step 0.1 (the reference example's wavelet, step and
    scaling) and a threshold from the data's noise level (the universal threshold; the
    example's 0.06 is reported beside it)."""
    from mripy_gb300 import operators as ops
    from mripy_gb300 import solvers
    from mripy_gb300.utilities import optscaling, universal_threshold
    nft = ops.NUFFT3d(wl.shape, tuning=tuning)
    nft.set_ktraj(*wl.coords)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nft.pipe_menon_dcf(20)
    torch.cuda.synchronize()
    t_dcf = time.perf_counter() - t0
    A = ops.joint2operators(ops.espirit(wl.sens), nft)
    x = torch.from_numpy(np.ascontiguousarray(wl.base_image).astype(np.complex64)).cuda()[..., None]
    y = A.forward(x)
    rng = np.random.default_rng(4)
    sigma = float(torch.linalg.vector_norm(y)) / np.sqrt(y.numel()) * 10 ** (-30 / 20)
    noise = torch.from_numpy((rng.standard_normal(tuple(y.shape)) + 1j * rng.standard_normal(tuple(y.shape)))
                             .astype(np.complex64) * sigma / np.sqrt(2)).cuda()
    y = y + noise
    W = solvers.DWTnd("haar", level=4, axes=(0, 1, 2))
    # the reference script divides the data by optscaling(Aopt, kdata) before the solver
    # (examples/pics_IST_3dute_wavelet_L1.py:79-80), so th is relative to the image peak
    scale = optscaling(A, y)
    y = y / scale
    adj = A.backward(y)
    # threshold for this data's noise level (the reference example's 0.06 belongs to its
    # own data): the universal threshold of the scaled adjoint image
    th = universal_threshold(adj, axes=(0, 1, 2))
    solvers.IST_wrap(A, W, y, 2, 0.1, th)              # warm-up (plans, iteration graph)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xr = solvers.IST_wrap(A, W, y, 30, 0.1, th)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    xt = x.reshape(-1)

    def err(v):
        xh = v.reshape(-1)
        a = torch.vdot(xh, xt) / torch.vdot(xh, xh)
        return round(float(torch.linalg.vector_norm(a * xh - xt) / torch.linalg.vector_norm(xt)), 4)
    return {"ist_iterations": 30, "wavelet": "haar level 4", "step": 0.1,
            "th": round(th, 4), "th_rule": "universal threshold sigma sqrt(2 ln N) of the scaled adjoint image "
                                          "(sigma: median finest diagonal Haar detail / 0.6745)",
            "ms_total": round(dt * 1e3, 2), "ms_per_iteration": round(dt * 1e3 / 30, 3),
            "includes": "A^H y with dcf, 1 prox, 29 x (normal operator + fused gradient/prox kernel)",
            "dcf": "Pipe-Menon, 20 iterations, %.1f ms" % (t_dcf * 1e3),
            "data_scaling": "kdata / optscaling(A, kdata) = kdata / %.4g" % scale,
            "rel_error_vs_phantom": err(xr), "rel_error_adjoint_only": err(adj),
            "rel_error_fista_30": err(solvers.FIST_wrap(A, W, y, 30, 0.1, th)),
            "rel_error_ist_30_reference_th_0.06": err(solvers.IST_wrap(A, W, y, 30, 0.1, 0.06)),
            "noise": "complex Gaussian, 30 dB SNR"}


def autograd_time(torch, wl, tuning, steps=20):
    """Differentiable NUFFT (the 16-coil spiral with perturbed float32 coordinates): loss =
    ||A(x; k) - y||^2 with y simulated on the unperturbed trajectory.  One step = forward (bin
    sort of the current trajectory, type-2) and backward (image gradient by the adjoint
    pipeline, trajectory gradient by pad + FFT + the weight-derivative interp kernel)."""
    from mripy_gb300 import autograd as AG
    from mripy_gb300 import synth
    from mripy_gb300.plan import NufftPlan
    cfg = synth.config5()
    plan = NufftPlan(2, wl.shape, n_coil=wl.n_coil, eps=wl.eps, tuning=tuning)
    img = torch.from_numpy(np.ascontiguousarray(cfg["image"])).cuda()[None]
    k_true = [torch.from_numpy(2 * np.pi * np.asarray(v, dtype=np.float64)).cuda() for v in cfg["k"]]
    y = plan.set_points(k_true).type2(img).detach()
    k = torch.from_numpy(np.stack([np.asarray(c, dtype=np.float32) for c in wl.coords])).cuda().requires_grad_(True)
    x = (img * 0.9).requires_grad_(True)

    def step():
        x.grad = None
        k.grad = None
        c = AG.nufft_forward(x, k, plan)
        loss = (c - y).abs().pow(2).sum()
        loss.backward()
        return loss

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        loss = step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    M, nc = wl.M, wl.n_coil
    return {"steps": steps, "ms_per_step": round(ms, 4), "value": round(M * nc / (ms * 1e-3) / 1e6, 2),
            "unit": UNIT, "loss": float(loss.detach()), "grad_k_rms": float(k.grad.pow(2).mean().sqrt()),
            "includes": "bin sort of the perturbed trajectory, type-2, loss, backward: image gradient "
                        "(type-1) and trajectory gradient (pad, FFT, weight-derivative interp)"}


def _centre(shape, n):
    return tuple(slice(m // 2 - n // 2, m // 2 - n // 2 + n) for m in shape)


def espirit_time(torch, wl, reps=5):
    """ESPIRiT coil maps (espirit/espirit_func.py) from the centre of the workload's fully
    sampled multi-coil k-space: 2-D 32^2 calibration region, 16^2 window; 3-D 24^3, 8^3.
    pad_before_espirit 0 (the reference default: eigen step on the calibration grid, maps
    interpolated by FFT) and, in 2-D, 1 (eigen step on every image pixel).  Beside the GPU
    time: the FP64 numpy restatement on the host (one run) and the maps' agreement with it;
    the eigen kernel alone is timed with CUDA events on the full-image case."""
    from mripy_gb300 import espirit as E
    from oracle import espirit_oracle as EO
    d = wl.dim
    axes = tuple(range(d))
    ksp = EO.ft_forward(wl.base_image[..., None] * wl.sens, axes)
    calib, win = (32, (16, 16)) if d == 2 else (24, (8, 8, 8))
    xcrop = np.ascontiguousarray(ksp[_centre(wl.shape, calib)]).astype(np.complex64)
    xc = torch.from_numpy(xcrop).cuda()
    x_shape = wl.shape + (wl.n_coil,)
    out = {"calibration": [calib] * d, "window": list(win), "coils": wl.n_coil}
    for pb in ((0, 1) if d == 2 else (0,)):
        E.espirit_nd(xc, x_shape, hkwin_shape=win, pad_before_espirit=pb)          # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            vg, sg, info = E.espirit_nd(xc, x_shape, hkwin_shape=win, pad_before_espirit=pb, return_info=True)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3 / reps
        t1 = time.perf_counter()
        vr, sr, _ = EO.espirit(xcrop.astype(np.complex128), x_shape, hkwin_shape=win, pad_before_espirit=pb,
                               return_info=True)
        s_cpu = time.perf_counter() - t1
        v = vg.cpu().numpy()
        s_map = sg.cpu().numpy()
        keep = sr > 0.05
        agree = np.abs(np.sum(v * np.conj(vr), axis=-1)) / (np.linalg.norm(v, axis=-1) * np.linalg.norm(vr, axis=-1)
                                                             + 1e-30)
        out["pad_before_espirit_%d" % pb] = {
            "ms_gpu": round(ms, 3), "s_cpu_fp64_port": round(s_cpu, 3), "cpu_cores": 1,
            "kept_singular_vectors": int(info["nsv"]),
            "eigen_pixels": int(np.prod(wl.shape)) if pb else calib ** d,
            "map_agreement_q01": round(float(np.quantile(agree[keep], 0.01)), 6),
            "eigenvalue_map_rel_err": float("%.2e" % (np.linalg.norm(s_map[keep] - sr[keep]) /
                                                      np.linalg.norm(sr[keep])))}
        if pb == 1:
            # the eigen kernel alone on the same shape: (pixels, kept vectors, coils)
            nsv = int(info["nsv"])
            a = torch.randn((int(np.prod(wl.shape)), nsv, wl.n_coil), dtype=torch.complex64, device="cuda")
            stream = torch.cuda.current_stream()
            flush_buf = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
            t_k, _ = event_time(torch, lambda: E.espirit_eigen(a), 10, stream, lambda: flush_buf.fill_(1.0))
            nbytes = a.numel() * 8
            out["eigen_kernel"] = {"ms": round(t_k, 4), "pixels": int(a.shape[0]), "nsv": nsv, "coils": wl.n_coil,
                                   "power_iterations": 64, "input_bytes": nbytes,
                                   "input_GBps": round(nbytes / (t_k * 1e-3) / 1e9, 1)}
    return out


def haar_time(torch, wl, level=4, reps=20):
    """Level-4 orthonormal Haar transform (mripy's DWTnd('haar') through pywt) over the
    spatial axes of the workload's image (the SENSE-combined image the IST solver
    thresholds) and of its coil stack (coils interleaved as the trailing axis): forward,
    inverse and the fused wavelet-L1 prox, each one kernel, timed with CUDA events (L2
    flushed between launches) against the measured HBM copy bandwidth; the FP64 numpy
    restatement on the host beside it."""
    from mripy_gb300 import plan as P
    from oracle import solver_oracle as SO
    axes = tuple(range(wl.dim))
    stream = torch.cuda.current_stream()
    flush_buf = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    flush = lambda: flush_buf.fill_(1.0)            # noqa: E731
    peak, peak_kind = peaks()
    out = {"level": level, "axes": list(axes), "peak": "%s %.0f GB/s" % (peak_kind, peak)}
    for case, shape in (("image", wl.shape), ("coil_stack", wl.shape + (wl.n_coil,))):
        g = torch.Generator(device="cuda").manual_seed(5)
        x = torch.randn(shape, dtype=torch.complex64, device="cuda", generator=g)
        c = torch.empty_like(x)
        y = torch.empty_like(x)
        nbytes = 2 * x.numel() * 8                   # read + write of the complex64 array
        res = {"shape": list(shape), "bytes_per_launch": nbytes}
        for name, fn in (("forward", lambda: P.haar_dwt(x, level, axes, out=c)),
                         ("inverse", lambda: P.haar_dwt(c, level, axes, inverse=True, out=y)),
                         ("prox", lambda: P.prox_haar(x, 0.1, level, axes, out=y))):
            fn()
            t, _ = event_time(torch, fn, reps, stream, flush)
            gbs = nbytes / (t * 1e-3) / 1e9
            res[name] = {"ms": round(t, 4), "GBps": round(gbs, 1), "frac_of_hbm": round(gbs / peak, 3)}
        xs = x.cpu().numpy().astype(np.complex128)
        t0 = time.perf_counter()
        ref = SO.haar_dwt(xs, level, axes)
        res["cpu_fp64_port_forward_s"] = round(time.perf_counter() - t0, 3)
        res["forward_rel_err_vs_port"] = float("%.2e" % (np.linalg.norm(c.cpu().numpy() - ref) / np.linalg.norm(ref)))
        out[case] = res
    return out


CPU_SUBSET_3D = 131072   # samples gridded per CPU step in 3-D (every coil); 2-D grids them all


def cpu_step(wl, workers):
    """One step of the reference's CPU NUFFT (the FP64 C restatement of mripy's
    build_grid_*_fast loops, OpenMP over the coils as mripy's prange, scipy.fft with
    ``workers`` threads standing in for pyFFTW) on group 0, every coil: deapodise + pad +
    FFT, interp, spread, inverse FFT + crop + deapodise.  2-D grids all of the group's
    samples.  3-D grids a strided subset of CPU_SUBSET_3D samples (whole 128-sample runs),
    the pad/FFT/crop stages run at full size, and the step time is extrapolated as
    t(pad, FFTs, crop) + t(interp + spread of the subset) x (samples / subset): the tap
    loops cost the same per sample wherever the sample lies.  Returns (value in Msamples/s
    counting every coil, seconds of the extrapolated step, description)."""
    import oracle as O
    from oracle import nufft_oracle as NO
    a, b = wl.offsets[0], wl.offsets[1]
    Mg, nc, d = b - a, wl.n_coil, wl.dim
    ns, nf, tau = NO._params_for(d, wl.shape, wl.eps)
    if d == 3 and Mg > CPU_SUBSET_3D:
        run = 128
        stride = max(1, Mg // CPU_SUBSET_3D)
        starts = np.arange(0, Mg - run + 1, run * stride)[:CPU_SUBSET_3D // run]
        sub = (starts[:, None] + np.arange(run)[None, :]).reshape(-1)
    else:
        sub = np.arange(Mg)
    xs_sub = tuple(np.ascontiguousarray(c[a:b][sub]) for c in wl.coords)
    img = wl.imgs[0].astype(np.complex128)
    axes = tuple(range(1, d + 1))
    t0 = time.perf_counter()
    Gk, _ = NO._type2_grid(img, wl.shape, nf, tau, 1, workers)               # deapod, pad, FFT
    t1 = time.perf_counter()
    c = O.interp(xs_sub, Gk, tau, ns)                                        # (coils, n)
    F = O.spread(xs_sub, c, tau, ns, nf)
    t2 = time.perf_counter()
    F = NO._fftn(F, axes, True, workers)
    F = NO._crop(F, wl.shape, nf) * NO._deapod(wl.shape, tau, d)[None] * (1.0 / Mg)
    t3 = time.perf_counter()
    t = (t1 - t0) + (t3 - t2) + (t2 - t1) * (Mg / len(sub))
    desc = ("%s: group 0, all %d coils, %s, fwd+adj; FP64 C restatement of build_grid_*_fast (OpenMP over "
            "coils as mripy's prange: %d threads) + scipy.fft with %d workers" % (
                wl.name, nc, ("all %d samples" % Mg) if len(sub) == Mg else
                ("tap loops on %d of %d samples (strided 128-sample runs), scaled to all; pad/FFT/crop at "
                 "full size" % (len(sub), Mg)), min(nc, os.cpu_count() or 1), workers))
    return Mg * nc / t / 1e6, t, desc


def run_reference(args, wl):
    """The reference arm: mripy's CPU NUFFT (the FP64 port of its loops) on the host cores,
    one bounded step per timed step, the same workload keys as the GPU arm's line."""
    from oracle import nufft_oracle as NO
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    cores = os.cpu_count() or 1
    workers = min(cores, 64)
    for _ in range(max(0, args.warmup)):
        cpu_step(wl, workers)
    t0 = time.perf_counter()
    vals = [cpu_step(wl, workers) for _ in range(args.steps)]
    wall = time.perf_counter() - t0
    value = float(np.mean([v[0] for v in vals]))
    ns, nf, _ = NO._params_for(wl.dim, wl.shape, wl.eps)
    cb = {"value": round(value, 4), "unit": UNIT, "kind": "port", "cores": workers,
          "gridding_threads": min(cores, wl.n_coil), "fft_workers": workers, "sample": vals[0][2],
          "seconds_per_step": round(float(np.mean([v[1] for v in vals])), 3)}
    return {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(float(np.mean([v[1] for v in vals])) * 1e3, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": line_config(wl, nf, ns, world), "impl": "reference",
            "reference_note": "mripy's NUFFT is Python+numba (not installable on the GPU host); timed as the FP64 "
                              "C restatement of its CPU loops (oracle/), on all host threads it can use",
            "cpu_baseline": cb,
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s_timed": round(wall, 2)}


def cpu_baseline_subprocess(wl):
    """The GPU arm's cpu_baseline: the reference arm's own measurement (one warm-up and one
    step), run in a fresh process so that the CPU figure does not depend on the GPU
    process's threads; both arms report the same quantity."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--workload", wl.name,
           "--steps", "1", "--warmup", "1"]
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    try:
        out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, check=True).stdout
        line = json.loads([ln for ln in out.splitlines() if ln.startswith("{")][-1])
        return line["cpu_baseline"]
    except Exception as exc:                     # the GPU figures stand without it
        return {"value": None, "unit": UNIT, "kind": "port", "cores": None,
                "sample": "reference-arm subprocess failed: %s" % str(exc)[:200]}


def step_kernels(torch, wl, coords, tuning, reps=3):
    """The NUFFT step alone (type-2 then type-1 over every instance, eager launches), run
    ``reps`` times after one warm-up, with each stage's CUDA-event time: the entry point for
    profiling the step's kernels without the rest of the benchmark."""
    from mripy_gb300 import _native as N
    from mripy_gb300.plan import NufftPlan
    dev = torch.device("cuda")
    plan = NufftPlan(wl.dim, wl.shape, n_coil=wl.n_coil, n_traj=wl.n_traj, eps=wl.eps, max_nspread=wl.max_nspread,
                     tuning=tuning)
    plan.set_points(coords, traj_offsets=wl.offsets)
    img = torch.from_numpy(np.ascontiguousarray(wl.imgs)).to(dev)
    samples = torch.empty((wl.M, wl.n_coil), dtype=torch.complex64, device=dev)
    out = torch.empty_like(img)
    grid = plan.grid()
    stream = torch.cuda.current_stream()
    stages = {"pad_deapod": lambda: plan.pad_deapod(img, grid),
              "fft": lambda: plan.fft_band(grid, N.GBN_FFT_FORWARD, N.GBN_BAND_INPUT),
              "interp": lambda: plan.interp(grid, out=samples), "spread": lambda: plan.spread(samples, grid),
              "fft_inverse": lambda: plan.fft_band(grid, N.GBN_FFT_INVERSE, N.GBN_BAND_OUTPUT),
              "crop_deapod": lambda: plan.crop_deapod(grid, out)}
    for f in stages.values():
        f()
    torch.cuda.synchronize()
    times = {k: [] for k in stages}
    for _ in range(reps):
        for k, f in stages.items():
            t, _ = event_time(torch, f, 1, stream)
            times[k].append(t)
    plan.status()
    info = plan.info()
    return {"ms": {k: round(float(np.median(v)), 4) for k, v in times.items()}, "spread_tile": list(info["spread_tile"]),
            "max_subproblem": info["max_subproblem"], "spread_kernels": info["spread_kernels"],
            "launches_per_run": "pad, FFT (cuFFT), interp, spread (+ split-tile zeroing, dense-tile instance), "
                                "inverse FFT, crop"}


def run_solver_only(args, wl):
    import torch
    coords = [torch.from_numpy(c).cuda() for c in wl.coords]
    tuning = None
    if args.tune == "auto":
        from mripy_gb300.tune import autotune
        tuning = autotune(wl.dim, wl.shape, coords, n_coil=wl.n_coil, n_traj=wl.n_traj, traj_offsets=wl.offsets,
                          eps=wl.eps, cache_file=args.tune_cache)
    if args.part == "step":
        return {"workload": wl.description, "part": "step", "step": step_kernels(torch, wl, coords, tuning)}
    if args.part == "autograd":
        return {"workload": wl.description, "part": "autograd", "autograd": autograd_time(torch, wl, tuning)}
    if args.part == "espirit":
        return {"workload": wl.description, "part": "espirit", "espirit": espirit_time(torch, wl)}
    if args.part == "haar":
        return {"workload": wl.description, "part": "haar", "haar": haar_time(torch, wl)}
    res = cg_sense_time(torch, wl, coords) if wl.name == "c2" else ist_time(torch, wl, tuning)
    return {"workload": wl.description, "part": "solver", "solver": res}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c4", choices=["c1", "c2", "c3", "c4", "c5"])
    ap.add_argument("--tune", default="auto", choices=["auto", "off"],
                    help="auto: the autotuner picks tiles / threads / coils per block on the workload's "
                         "trajectory before the timed region; off: library defaults")
    ap.add_argument("--tune-cache", default=None,
                    help="JSON file of autotuner results: read if it holds this workload's key, else "
                         "written; lets a profiler run reuse the tiling of an earlier run")
    ap.add_argument("--part", default="all", choices=["all", "step", "solver", "autograd", "espirit", "haar"],
                    help="step: only the NUFFT step's stages, eager, 3 runs (for profiling); "
                         "solver: only the solver timing of c2 (CG-SENSE) or c4 (IST); autograd: only "
                         "the differentiable step of c5; espirit: ESPIRiT maps from c2's or c4's coil "
                         "k-space; haar: the Haar transform and prox on c2's or c4's coil stack; one "
                         "JSON line with its figures (for profiling)")
    args = ap.parse_args()
    if args.part != "all":
        ok = {"step": ("c1", "c2", "c3", "c4", "c5"), "solver": ("c2", "c4"), "autograd": ("c5",),
              "espirit": ("c2", "c4"), "haar": ("c2", "c4")}[args.part]
        if args.workload not in ok or args.impl != "gb300":
            ap.error("--part %s takes --workload %s with the gb300 arm" % (args.part, " or ".join(ok)))
        from mripy_gb300 import build
        build.build()
        print(json.dumps(run_solver_only(args, make_workload(args.workload))))
        return
    if args.impl == "gb300":
        args.warmup = max(args.warmup, 3)
    import oracle
    oracle.build()
    wl = make_workload(args.workload)
    if args.impl == "reference":
        res = run_reference(args, wl)
    else:
        from mripy_gb300 import build
        build.build()
        res = run_gpu(args, wl)
    if res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
