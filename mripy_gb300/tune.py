"""Autotuner: pick tile sizes, threads per block and work-item size per trajectory.

The gridding kernels' best tiling depends on the sample density: dense k-space centres
want small work items (more blocks, less imbalance), sparse trajectories want larger
tiles (fewer halo duplicates).  ``autotune`` times candidate ``Tuning``s on the caller's
own trajectory with CUDA events (spread and interp separately, so the search is additive
rather than a full product) and returns the fastest; results are cached per problem key
(dimension, image shape, coils, groups, eps, sample count and a coarse density signature).

    tuning = autotune(2, (256, 256), [x, y], n_coil=8, eps=5e-6)
    plan = NufftPlan(2, (256, 256), n_coil=8, eps=5e-6, tuning=tuning)
"""
import json
import os

import numpy as np
import torch

from .plan import NufftPlan, Tuning

_CACHE = {}


def _spread_candidates(dim, n_coil):
    """(tile, threads, coil_group, spread_variant) tuples: the register-tile kernels' own
    tiles (rows of 4 per warp, 4 columns per lane) for 4 and 8 coils per block, in 3-D with 8
    coils also the tensor-core kernel's 4 x 8 x 16 tile and the cube kernel's tiles (8 or 16
    cubes of 4^3 cells), plus shared-memory tiles."""
    out = []
    groups = [cg for cg in (8, 4) if n_coil >= cg]
    if dim == 2:
        for cg in groups:
            for th in (128, 256):
                out.append(((4 * th // 32, 4 * 32 // cg), th, cg, 0))
        out += [((16, 32), 256, 8, 0), ((32, 32), 256, 8, 0)]
        if n_coil < 4:
            # one-coil plans (the plain per-instance path): 128-thread blocks measured best
            out += [((16, 32), 128, 8, 0), ((32, 32), 128, 8, 0)]
    elif dim == 3:
        for cg in groups:
            for th in (128, 256):
                rows = 4 * th // 32
                for ty in (4, 8, 16):
                    if rows % ty == 0:
                        out.append(((rows // ty, ty, 4 * 32 // cg), th, cg, 1 if cg == 8 else 0))
        if n_coil >= 8:
            out.append(((4, 8, 16), 256, 8, 3))
            for tile in ((8, 8, 8), (4, 8, 16), (8, 8, 16), (16, 8, 8)):
                out.append((tile, 256, 8, 2))
        out += [((8, 8, 32), 256, 8, 0)]
    else:
        out = [((t,), 256, 8, 0) for t in (1024, 512, 2048)]
    return out


def _interp_threads(dim):
    return (256, 512) if dim == 2 else (128, 256)


def _interp_coil_groups(n_coil):
    return [0] + [cg for cg in (8, 4, 2) if cg <= n_coil]


def candidate_tunings(dim, n_coil):
    """Every configuration the search below can time: the spread candidates, then the interp
    ones (each with the other kernel at library defaults)."""
    _, interp_c = _candidates(dim)
    out = [Tuning(spread_tile=t, threads=th, coil_group=cg, spread_variant=v)
           for t, th, cg, v in _spread_candidates(dim, n_coil)]
    out += [Tuning(interp_tile=t, interp_threads=th, interp_coil_group=cg)
            for t in interp_c for th in _interp_threads(dim) for cg in _interp_coil_groups(n_coil)]
    return out


def _candidates(dim):
    if dim == 2:
        spread = [(16, 32), (8, 32), (32, 32), (16, 64), (32, 16)]
        interp = [(16, 16), (8, 32), (16, 32), (8, 16), (32, 32)]
    elif dim == 3:
        spread = [(8, 8, 32), (8, 8, 16), (4, 8, 32), (8, 16, 16)]
        # (8, 8, 8), (16, 8, 8), (8, 4, 8): planes the plane-streaming kernel takes at 8 coils
        interp = [(8, 8, 8), (16, 8, 8), (8, 4, 8), (4, 8, 16), (8, 8, 16), (4, 4, 16)]
    else:
        spread = [(1024,), (512,), (2048,)]
        interp = [(1024,), (512,), (256,)]
    return spread, interp


def density_signature(coords, bins=8):
    """log2 of (peak / mean) sample count over a coarse bins^dim histogram of the wrapped
    coordinates: 0 for uniform sampling, large for radial/spiral centres."""
    pts = [torch.remainder(c.detach().double(), 2 * np.pi) for c in coords]
    idx = torch.zeros_like(pts[0], dtype=torch.int64)
    for p in pts:
        idx = idx * bins + torch.clamp((p / (2 * np.pi) * bins).long(), 0, bins - 1)
    counts = torch.bincount(idx, minlength=bins ** len(coords)).double()
    mean = counts.mean().item()
    return int(round(np.log2(max(counts.max().item(), 1.0) / max(mean, 1e-9))))


def _key(dim, shape, n_coil, n_traj, eps, M, sig):
    return "d%d_%s_c%d_g%d_e%.0e_m%d_s%d" % (dim, "x".join(map(str, shape)), n_coil, n_traj, eps,
                                             int(np.log2(max(M, 1))), sig)


def _time(fn, reps):
    flush = torch.empty(64 * 2 ** 20, dtype=torch.float32, device="cuda")
    ts = []
    for _ in range(reps):
        flush.fill_(1.0)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b))
    return float(np.median(ts))


def _measure(dim, shape, coords, n_coil, n_traj, traj_offsets, eps, tuning, reps):
    p = NufftPlan(dim, shape, n_coil=n_coil, n_traj=n_traj, eps=eps, tuning=tuning,
                  max_nspread=6 if dim == 3 else None)
    try:
        p.set_points(coords, traj_offsets=traj_offsets)
        g = torch.randn(p.grid().shape, dtype=torch.complex64, device="cuda")
        s = p.empty_samples()
        t_i = _time(lambda: p.interp(g, out=s), reps)
        t_s = _time(lambda: p.spread(s, g), reps)
        return t_s, t_i
    finally:
        p.close()


def autotune(dim, shape, coords, n_coil=1, n_traj=1, traj_offsets=None, eps=5e-6, reps=5, cache_file=None,
             verbose=False):
    """Return the fastest ``Tuning`` for this trajectory (see module docstring)."""
    coords = [c if isinstance(c, torch.Tensor) else torch.as_tensor(np.asarray(c)) for c in coords]
    coords = [c.to("cuda") for c in coords]
    M = coords[0].numel()
    key = _key(dim, tuple(shape), n_coil, n_traj, eps, M, density_signature(coords))
    if key in _CACHE:
        return _CACHE[key]
    if cache_file and os.path.exists(cache_file):
        with open(cache_file) as f:
            stored = json.load(f)
        if key in stored:
            t = Tuning(**stored[key])
            _CACHE[key] = t
            return t
    _, interp_c = _candidates(dim)
    best_s = best_i = None
    # spread tiling (interp at default), then interp tiling (spread at the winner)
    for tile, th, cg, var in _spread_candidates(dim, n_coil):
        # the cube and tensor-core kernels need long work items to keep their rings full:
        # time them at 2048
        tu = Tuning(spread_tile=tile, threads=th, coil_group=cg, spread_variant=var,
                    max_subproblem=2048 if var >= 2 else 0)
        try:
            t_s, _ = _measure(dim, shape, coords, n_coil, n_traj, traj_offsets, eps, tu, reps)
        except Exception:
            continue
        if verbose:
            print("spread", tile, th, cg, var, t_s)
        if best_s is None or t_s < best_s[0]:
            best_s = (t_s, tile, th, cg, var)
    icg = _interp_coil_groups(n_coil)
    for tile in interp_c:
        for th in _interp_threads(dim):
            for cg in icg:
                tu = Tuning(interp_tile=tile, interp_threads=th, interp_coil_group=cg)
                try:
                    _, t_i = _measure(dim, shape, coords, n_coil, n_traj, traj_offsets, eps, tu, reps)
                except Exception:
                    continue
                if verbose:
                    print("interp", tile, th, cg, t_i)
                if best_i is None or t_i < best_i[0]:
                    best_i = (t_i, tile, th, cg)
    if best_s is None or best_i is None:
        raise RuntimeError("no tuning candidate ran")
    best = None
    for ms in ((1024, 2048, 4096, 8192) if best_s[4] >= 2 else (64, 128, 256, 512, 1024)):
        tu = Tuning(spread_tile=best_s[1], threads=best_s[2], coil_group=best_s[3], interp_tile=best_i[1],
                    interp_threads=best_i[2], interp_coil_group=best_i[3], max_subproblem=ms,
                    spread_variant=best_s[4])
        t_s, t_i = _measure(dim, shape, coords, n_coil, n_traj, traj_offsets, eps, tu, reps)
        if verbose:
            print("max_subproblem", ms, t_s + t_i)
        if best is None or t_s + t_i < best[0]:
            best = (t_s + t_i, tu)
    tuning = best[1]
    _CACHE[key] = tuning
    if cache_file:
        stored = {}
        if os.path.exists(cache_file):
            with open(cache_file) as f:
                stored = json.load(f)
        stored[key] = {"spread_tile": list(tuning.spread_tile), "interp_tile": list(tuning.interp_tile),
                       "max_subproblem": tuning.max_subproblem, "coil_group": tuning.coil_group,
                       "threads": tuning.threads, "interp_threads": tuning.interp_threads,
                       "interp_coil_group": tuning.interp_coil_group, "spread_variant": tuning.spread_variant}
        with open(cache_file, "w") as f:
            json.dump(stored, f, indent=1)
    return tuning
