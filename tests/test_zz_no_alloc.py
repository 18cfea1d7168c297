"""gbn_spread2d_noalloc, the allocation-free 2-D spread, against the FP64 oracle and the
plan-based gbn_spread.

Callers that cannot allocate device memory (a framework owning the GPU memory pool,
real-time loops that must not block in cudaMalloc, plugin hosts that pass pre-sized
buffers) use gbn_spread2d_noalloc: its binning scratch is a fixed device array inside the
library.  This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.

Tolerance: TOL = 2e-5 relative L2, the GPU parity bar (complex64 samples and FP32
accumulation against the FP64 oracle, or against gbn_spread's different summation order).
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O
from mripy_gb300 import _native as N
from mripy_gb300.plan import NufftPlan

pytestmark = pytest.mark.gpu

TOL = 2e-5
MAX_SAMPLES = 262144      # GBN_NOALLOC_MAX_SAMPLES
MAX_TILES = 16384         # GBN_NOALLOC_MAX_TILES


def _rel(a, b):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else a
    b = b.cpu().numpy() if isinstance(b, torch.Tensor) else b
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _noalloc(x, y, c, n_coil, shape, eps, out):
    lib = N.lib()
    L = N.Layout(0, c.stride(1), c.stride(0))
    dt = N.GBN_COORD_F64 if x.dtype == torch.float64 else N.GBN_COORD_F32
    return lib.gbn_spread2d_noalloc(dt, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), x.numel(),
                                    ctypes.c_void_p(c.data_ptr()), L, n_coil, shape[0], shape[1], eps, 1.0,
                                    ctypes.c_void_p(out.data_ptr()),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def _oracle_spread(xs, c, shape, eps):
    """FP64 gridding sum (build_grid_2d1_fast) of the samples c (M, n_coil) at xs (2, M)."""
    ns, nf, tau = O.grid_params(2, shape[0], shape[1], eps=eps)
    return O.spread((xs[0], xs[1]), c.T.astype(np.complex128), tau, ns, nf)


def _case(rng, M, n_coil, dense_frac=1 / 3, dense_scale=0.05):
    xs = rng.uniform(-np.pi, np.pi, (2, M))
    xs[:, : int(M * dense_frac)] *= dense_scale          # a dense centre: split tiles
    c = (rng.standard_normal((M, n_coil)) + 1j * rng.standard_normal((M, n_coil))).astype(np.complex64)
    return xs, c


@pytest.mark.parametrize("n_coil", [1, 4, 8, 9])
@pytest.mark.parametrize("coord_dtype", [np.float64, np.float32])
def test_noalloc_spread_matches_oracle_and_plan_on_two_calls(n_coil, coord_dtype):
    rng = np.random.default_rng(40 + n_coil)
    shape, eps = (96, 80), 5e-6
    tdt = torch.float64 if coord_dtype == np.float64 else torch.float32
    # two calls in a row with different trajectories, sizes and samples: the shared
    # scratch array must be re-initialised by each call
    for M in (60000, 23456):
        xs, cn = _case(rng, M, n_coil)
        xs = xs.astype(coord_dtype)
        x = torch.from_numpy(xs[0]).cuda()
        y = torch.from_numpy(xs[1]).cuda()
        c = torch.from_numpy(cn).cuda()
        plan = NufftPlan(2, shape, n_coil=n_coil, eps=eps).set_points([x, y])
        ref = plan.spread(c, grid=plan.grid()).clone()
        plan.close()
        out = torch.full_like(ref, float("nan"))        # every cell must be written
        assert x.dtype == tdt
        assert _noalloc(x, y, c, n_coil, shape, eps, out) == 0, N.last_error()
        torch.cuda.synchronize()
        assert torch.isfinite(torch.view_as_real(out)).all()
        orc = _oracle_spread(xs.astype(np.float64), cn, shape, eps)
        assert _rel(out, orc) < TOL
        assert _rel(out, ref) < TOL


def test_noalloc_allocates_nothing():
    """After a warm-up call (which resolves the array and loads the kernels), further calls
    leave the device's free memory unchanged."""
    rng = np.random.default_rng(41)
    shape, eps, n_coil = (96, 80), 5e-6, 8
    xs, cn = _case(rng, 50000, n_coil)
    x = torch.from_numpy(xs[0]).cuda()
    y = torch.from_numpy(xs[1]).cuda()
    c = torch.from_numpy(cn).cuda()
    out = torch.empty((n_coil, 192, 160), dtype=torch.complex64, device="cuda")
    assert _noalloc(x, y, c, n_coil, shape, eps, out) == 0, N.last_error()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert _noalloc(x, y, c, n_coil, shape, eps, out) == 0, N.last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert _rel(out, _oracle_spread(xs, cn, shape, eps)) < TOL


def test_noalloc_at_its_limits():
    """GBN_NOALLOC_MAX_SAMPLES samples, nine tenths of them inside one 16 x 32 tile (so that
    tile splits into the most work items), on a grid of exactly GBN_NOALLOC_MAX_TILES tiles."""
    rng = np.random.default_rng(42)
    shape, eps = (1024, 2048), 5e-6               # nf 2048 x 4096 = 128 x 128 tiles of 16 x 32
    ns, nf, _ = O.grid_params(2, shape[0], shape[1], eps=eps)
    assert (nf[0] // 16) * (nf[1] // 32) == MAX_TILES
    M = MAX_SAMPLES
    xs = rng.uniform(-np.pi, np.pi, (2, M))
    h = 2 * np.pi / np.asarray(nf, dtype=np.float64)
    n_in = int(M * 0.9)
    # in tile (64, 64): cells x 1024..1039, y 2048..2079, away from its edges by the stencil
    xs[0, :n_in] = (1024 + ns + rng.uniform(0, 16 - 2 * ns, n_in)) * h[0]
    xs[1, :n_in] = (2048 + ns + rng.uniform(0, 32 - 2 * ns, n_in)) * h[1]
    cn = (rng.standard_normal((M, 1)) + 1j * rng.standard_normal((M, 1))).astype(np.complex64)
    x = torch.from_numpy(xs[0]).cuda()
    y = torch.from_numpy(xs[1]).cuda()
    c = torch.from_numpy(cn).cuda()
    out = torch.full((1,) + tuple(nf), float("nan"), dtype=torch.complex64, device="cuda")
    assert _noalloc(x, y, c, 1, shape, eps, out) == 0, N.last_error()
    torch.cuda.synchronize()
    assert torch.isfinite(torch.view_as_real(out)).all()
    assert _rel(out, _oracle_spread(xs, cn, shape, eps)) < TOL


def test_noalloc_leaves_out_non_finite_samples():
    rng = np.random.default_rng(43)
    shape, eps, n_coil = (96, 80), 5e-6, 2
    xs, cn = _case(rng, 30000, n_coil)
    bad = rng.choice(30000, 300, replace=False)
    xs[0, bad[:100]] = np.nan
    xs[1, bad[100:200]] = np.inf
    xs[0, bad[200:]] = -np.inf
    x = torch.from_numpy(xs[0]).cuda()
    y = torch.from_numpy(xs[1]).cuda()
    c = torch.from_numpy(cn).cuda()
    out = torch.full((n_coil, 192, 160), float("nan"), dtype=torch.complex64, device="cuda")
    assert _noalloc(x, y, c, n_coil, shape, eps, out) == 0, N.last_error()
    torch.cuda.synchronize()
    keep = np.ones(30000, dtype=bool)
    keep[bad] = False
    assert torch.isfinite(torch.view_as_real(out)).all()
    assert _rel(out, _oracle_spread(xs[:, keep], cn[keep], shape, eps)) < TOL


def test_noalloc_rejects_sizes_beyond_its_limits():
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    c = torch.zeros((8, 1), dtype=torch.complex64, device="cuda")
    out = torch.zeros((1, 192, 160), dtype=torch.complex64, device="cuda")
    lib = N.lib()
    L = N.Layout(0, 1, 1)
    p = ctypes.c_void_p
    st = lib.gbn_spread2d_noalloc(N.GBN_COORD_F64, p(x.data_ptr()), p(x.data_ptr()), MAX_SAMPLES + 1,
                                  p(c.data_ptr()), L, 1, 96, 80, 5e-6, 1.0, p(out.data_ptr()), None)
    assert st == 6 and "262144" in N.last_error()
    st = lib.gbn_spread2d_noalloc(N.GBN_COORD_F64, p(x.data_ptr()), p(x.data_ptr()), 8, p(c.data_ptr()), L, 1,
                                  95, 80, 5e-6, 1.0, p(out.data_ptr()), None)
    assert st == 6 and "whole" in N.last_error()
    st = lib.gbn_spread2d_noalloc(N.GBN_COORD_F64, p(x.data_ptr()), p(x.data_ptr()), 8, p(c.data_ptr()), L, 1,
                                  1024, 2064, 5e-6, 1.0, p(out.data_ptr()), None)
    assert st == 6 and "16384" in N.last_error()      # 128 x 129 tiles
