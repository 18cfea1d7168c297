"""Benchmark: batched NUFFT forward + adjoint Msamples/s on the batched 2-D multi-coil
workload (256^2 image x 8 coils, golden-angle radial 402 spokes x 512 samples,
oversampled grid 512^2, nspread 6).

One step = type-2 (forward) + type-1 (adjoint) over all 8 coils, replayed from one
CUDA graph; value = (samples x coils) / step time.  Also reported:
  plain       the per-instance path: one single-coil plan, eager launches, coil by coil
  e2e         the same step through the C ABI with host (pinned) buffers, H2D and D2H
              inside the timed region (gbn_type2_host + gbn_type1_host)
  roofline    dominant gridding kernel: algorithmic bytes / its CUDA-event duration vs
              the measured HBM copy bandwidth; fp32 fraction beside it
  cpu_baseline  the FP64 C restatement of mripy's CPU NUFFT on the host cores
  accuracy    relative L2 error vs the FP64 NUDFT on a sample subset

--impl reference times mripy's CPU NUFFT algorithm (the oracle port; mripy itself is
Python/numba and is not installed on the GPU host) on the same workload.
Under torchrun (N > 1) every rank runs its own replica (weak scaling, no collective
in the data path); rank 0 prints the line with the max step time over ranks.
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
WORKLOAD = "2-D 8-coil golden-angle radial 402x512 samples, 256^2 image, 512^2 grid, nspread 6 (eps 5e-6)"
UNIT = "Msamples/s"
L2_BYTES = 129 * 2 ** 20


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
        sm, smax, reasons, all_sm = [], 0.0, set(), []
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
            all_sm.append(mhz)
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


# ------------------------------------------------------------------------------ workload

def make_workload(torch):
    from mripy_gb300 import synth
    cfg = synth.config2()
    kx, ky = cfg["k"]
    x = 2 * np.pi * kx
    y = 2 * np.pi * ky
    imgs = (cfg["image"][..., None] * cfg["sens"]).astype(np.complex64)       # (256, 256, 8) coil images
    return x, y, imgs


def algorithmic_bytes(M, n_coil, dim, grid_cells):
    """Per direction: samples (complex64) + packed coordinates read once per shared
    trajectory (4 B per dim) + the oversampled grid of every coil (complex64)."""
    return 8 * M * n_coil + 4 * dim * M + 8 * grid_cells * n_coil


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


def run_gpu(args):
    import torch
    from mripy_gb300 import _native as N
    from mripy_gb300.plan import NufftPlan

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    x, y, imgs = make_workload(torch)
    M, n_coil, shape = len(x), imgs.shape[-1], imgs.shape[:2]
    xd = torch.from_numpy(x).to(dev)
    yd = torch.from_numpy(y).to(dev)
    img = torch.from_numpy(imgs).to(dev)[None]                              # (1, 256, 256, 8)
    samples = torch.empty((M, n_coil), dtype=torch.complex64, device=dev)
    out_img = torch.empty_like(img)
    plan = NufftPlan(2, shape, n_coil=n_coil, eps=5e-6).set_points([xd, yd])
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
    step_ms_med, step_ms = event_time(torch, g.replay, args.steps, stream, flush)
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
              "data": "synthetic (seeded phantom x coil maps, golden-angle radial trajectory)",
              "config": {"workload": WORKLOAD, "samples_per_coil": M, "coils": n_coil, "image": list(shape),
                         "grid": list(info["nf"]), "nspread": info["nspread"],
                         "step": "type-2 + type-1 over all coils, one CUDA graph",
                         "l2": "flushed between timed steps (write of %d MiB)" % (2 * L2_BYTES // 2 ** 20),
                         "parallelism": "replicas" if world > 1 else "single GPU"},
              "wall_s_timed": round(t_wall, 3)}
    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return None

    # --- per-kernel timing (gridding stages alone, same stream, L2 flushed)
    grid = plan.grid()
    plan.pad_deapod(img, grid)
    plan.fft(grid, N.GBN_FFT_FORWARD)
    grid_copy = grid.clone()
    t_interp, _ = event_time(torch, lambda: plan.interp(grid_copy, out=samples), 20, stream, flush)
    t_spread, _ = event_time(torch, lambda: plan.spread(samples, grid), 20, stream, flush)
    t_pad, _ = event_time(torch, lambda: plan.pad_deapod(img, grid), 20, stream, flush)
    t_fft, _ = event_time(torch, lambda: plan.fft(grid, N.GBN_FFT_FORWARD), 20, stream, flush)
    t_crop, _ = event_time(torch, lambda: plan.crop_deapod(grid, out_img), 20, stream, flush)
    G = info["grid_cells"]
    bytes_dir = algorithmic_bytes(M, n_coil, 2, G)
    fl = flops(M, n_coil, 2 * info["nspread"], 2)
    hbm, peak_kind = peaks()
    dominant = "spread" if t_spread >= t_interp else "interp"
    t_dom = max(t_spread, t_interp)
    achieved = bytes_dir / (t_dom * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "ncu_traffic_c2.txt")
    if os.path.exists(tpath):
        for ln in open(tpath):
            if ln.startswith(dominant + "_dram_bytes_per_launch:"):
                traffic = int(ln.split(":")[1])
    result["roofline"] = {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1),
                          "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 4), "traffic": traffic,
                          "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                          else "fallback 6.8 TB/s",
                          "algorithmic_bytes_per_launch": bytes_dir,
                          "fp32_tflops_achieved": round(fl / (t_dom * 1e-3) / 1e12, 2)}
    result["kernels_ms"] = {"interp": round(t_interp, 4), "spread": round(t_spread, 4), "pad_deapod": round(t_pad, 4),
                            "fft": round(t_fft, 4), "crop_deapod": round(t_crop, 4)}
    result["gpu_launches"] = 5 * args.steps  # pad, interp, zero-split, spread, crop per step (cuFFT not counted)

    # --- plain per-instance path: single-coil plan, eager, coil by coil
    p1 = NufftPlan(2, shape, n_coil=1, eps=5e-6).set_points([xd, yd])
    s1 = torch.empty((M, 1), dtype=torch.complex64, device=dev)
    o1 = torch.empty((1,) + tuple(shape) + (1,), dtype=torch.complex64, device=dev)
    coil_imgs = [img[..., c:c + 1].contiguous() for c in range(n_coil)]

    def plain_step():
        for c in range(n_coil):
            p1.type2(coil_imgs[c], out=s1)
            p1.type1(s1, out=o1)

    for _ in range(3):
        plain_step()
    t_plain, _ = event_time(torch, plain_step, min(100, max(5, args.steps // 2)), stream, flush)
    result["plain"] = {"value": round(M * n_coil / (t_plain * 1e-3) / 1e6, 2), "unit": UNIT,
                       "ms_per_step": round(t_plain, 4), "speedup_batched_vs_plain": round(t_plain / mean_ms, 2)}

    # --- accuracy vs FP64 NUDFT on a subset
    import oracle as O
    plan.type2(img, out=samples)
    plan.type1(samples, out=out_img)
    torch.cuda.synchronize()
    rng = np.random.default_rng(1)
    sub = rng.choice(M, 512, replace=False)
    cf = samples.cpu().numpy()
    ex = O.nudft_type2((x[sub], y[sub]), imgs[..., :2].astype(np.complex128), tuple(shape))
    err_fwd = np.linalg.norm(cf[sub, :2] - ex) / np.linalg.norm(ex)
    pix = rng.choice(shape[0] * shape[1], 256, replace=False)
    cs = cf[:, :1].astype(np.complex128)
    exa = O.nudft_type1((x, y), cs, tuple(shape), pixels=pix)[:, 0]
    ga = out_img[0, ..., 0].cpu().numpy().reshape(-1)[pix]
    err_adj = np.linalg.norm(ga - exa) / np.linalg.norm(exa)
    result["accuracy"] = {"fwd_rel_l2_vs_nudft": float("%.3e" % err_fwd), "adj_rel_l2_vs_nudft": float("%.3e" % err_adj),
                          "target": 1e-4}

    # --- end to end through the C ABI with pinned host buffers
    h_img = torch.from_numpy(imgs.reshape(1, *imgs.shape)).pin_memory()
    h_k = torch.empty((M, n_coil), dtype=torch.complex64).pin_memory()
    h_out = torch.empty_like(h_img).pin_memory()
    lib = N.lib()
    sp = ctypes.c_void_p(stream.cuda_stream)

    def e2e_step():
        N.check(lib.gbn_type2_host(plan._h, ctypes.c_void_p(h_img.data_ptr()), ctypes.c_void_p(h_k.data_ptr()), sp))
        N.check(lib.gbn_type1_host(plan._h, ctypes.c_void_p(h_k.data_ptr()), ctypes.c_void_p(h_out.data_ptr()), sp))

    for _ in range(3):
        e2e_step()
    ts = []
    for _ in range(min(50, max(5, args.steps))):
        flush()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        ts.append(time.perf_counter() - t0)
    t_e2e = float(np.mean(ts))
    img_bytes = imgs.nbytes
    k_bytes = M * n_coil * 8
    result["e2e"] = {"value": round(M * n_coil / t_e2e / 1e6, 2), "unit": UNIT,
                     "h2d_bytes_per_step": img_bytes + k_bytes, "d2h_bytes_per_step": k_bytes + img_bytes,
                     "ms_per_step": round(t_e2e * 1e3, 3),
                     "path": "gbn_type2_host + gbn_type1_host (host pinned buffers, includes H2D and D2H)"}

    # --- CPU baseline: FP64 port of mripy's CPU NUFFT on the host cores (bounded sample)
    result["cpu_baseline"] = cpu_baseline(x, y, imgs, sample_coils=n_coil, reps=1)
    if clocks:
        result["clocks"] = clocks
    if world > 1:
        torch.distributed.barrier()
    return result


def cpu_baseline(x, y, imgs, sample_coils, reps=1):
    import oracle as O
    cores = os.cpu_count() or 1
    workers = min(cores, 64)
    shape = imgs.shape[:2]
    sub = imgs[..., :sample_coils].astype(np.complex128)
    O.nufft_type2((x[:1000], y[:1000]), sub[..., :1], shape, eps=5e-6)         # load the library
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        c = O.nufft_type2((x, y), sub, shape, eps=5e-6, workers=workers)
        O.nufft_type1((x, y), c, shape, eps=5e-6, workers=workers)
        ts.append(time.perf_counter() - t0)
    t = float(np.median(ts))
    return {"value": round(len(x) * sample_coils / t / 1e6, 3), "unit": UNIT, "kind": "port",
            "cores": min(cores, sample_coils),
            "sample": "full workload, %d coils, fwd+adj, FP64 C restatement of build_grid_2d{1,2}_fast "
                      "(OpenMP over coils as mripy's prange) + scipy.fft with %d workers; %d rep(s)" % (
                          sample_coils, workers, reps),
            "seconds": round(t, 3)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    from mripy_gb300 import synth
    cfg = synth.config2()
    kx, ky = cfg["k"]
    x, y = 2 * np.pi * kx, 2 * np.pi * ky
    imgs = (cfg["image"][..., None] * cfg["sens"]).astype(np.complex64)
    n_coil = imgs.shape[-1]
    for _ in range(max(0, args.warmup)):
        cpu_baseline(x, y, imgs, n_coil, reps=1)
    t0 = time.perf_counter()
    vals = [cpu_baseline(x, y, imgs, n_coil, reps=1) for _ in range(args.steps)]
    wall = time.perf_counter() - t0
    secs = float(np.mean([v["seconds"] for v in vals]))
    value = len(x) * n_coil / secs / 1e6
    cb = dict(vals[0])
    cb["value"] = round(value, 3)
    return {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(secs * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": WORKLOAD}, "impl": "reference",
            "reference_note": "mripy's NUFFT is Python+numba (not installable on the GPU host); timed as the FP64 "
                              "C restatement of its CPU loops (oracle/), on all host threads it can use",
            "cpu_baseline": cb,
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s_timed": round(wall, 2)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    import oracle
    oracle.build()
    if args.impl == "reference":
        res = run_reference(args)
    else:
        from mripy_gb300 import build
        build.build()
        res = run_gpu(args)
    if res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
