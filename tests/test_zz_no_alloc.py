"""gbn_spread2d_noalloc, the allocation-free 2-D spread, against the plan-based gbn_spread.

Callers that cannot allocate device memory (a framework owning the GPU memory pool,
real-time loops that must not block in cudaMalloc, plugin hosts that pass pre-sized
buffers) use gbn_spread2d_noalloc: its binning scratch is a fixed device array inside the
library.  This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from mripy_gb300 import _native as N
from mripy_gb300.plan import NufftPlan

pytestmark = pytest.mark.gpu

TOL = 2e-5  # the GPU parity tolerance: FP32 summation order differs between the two paths


def _rel(a, b):
    return float((a - b).norm() / b.norm())


def _noalloc(x, y, c, n_coil, shape, eps, out):
    lib = N.lib()
    L = N.Layout(0, c.stride(1), c.stride(0))
    st = lib.gbn_spread2d_noalloc(N.GBN_COORD_F64, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                  x.numel(), ctypes.c_void_p(c.data_ptr()), L, n_coil, shape[0], shape[1], eps, 1.0,
                                  ctypes.c_void_p(out.data_ptr()),
                                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st


def test_noalloc_spread_matches_plan_spread_on_two_calls():
    rng = np.random.default_rng(40)
    shape, n_coil, eps = (96, 80), 3, 5e-6
    # two calls in a row with different trajectories, sizes and samples: the shared
    # scratch array must be re-initialised by each call
    for M in (60000, 23456):
        xs = rng.uniform(-np.pi, np.pi, (2, M))
        xs[:, : M // 3] *= 0.05                         # a dense centre: split tiles
        x = torch.from_numpy(xs[0]).cuda()
        y = torch.from_numpy(xs[1]).cuda()
        c = torch.from_numpy((rng.standard_normal((M, n_coil)) + 1j * rng.standard_normal((M, n_coil)))
                             .astype(np.complex64)).cuda()
        plan = NufftPlan(2, shape, n_coil=n_coil, eps=eps).set_points([x, y])
        ref = plan.spread(c, grid=plan.grid()).clone()
        out = torch.full_like(ref, float("nan"))        # every cell must be written
        assert _noalloc(x, y, c, n_coil, shape, eps, out) == 0, N.last_error()
        torch.cuda.synchronize()
        assert torch.isfinite(torch.view_as_real(out)).all()
        assert _rel(out, ref) < TOL
        plan.close()


def test_noalloc_rejects_sizes_beyond_its_limits():
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    c = torch.zeros((8, 1), dtype=torch.complex64, device="cuda")
    out = torch.zeros((1, 192, 160), dtype=torch.complex64, device="cuda")
    lib = N.lib()
    L = N.Layout(0, 1, 1)
    p = ctypes.c_void_p
    st = lib.gbn_spread2d_noalloc(N.GBN_COORD_F64, p(x.data_ptr()), p(x.data_ptr()), 262145, p(c.data_ptr()), L, 1,
                                  96, 80, 5e-6, 1.0, p(out.data_ptr()), None)
    assert st == 6 and "262144" in N.last_error()
    st = lib.gbn_spread2d_noalloc(N.GBN_COORD_F64, p(x.data_ptr()), p(x.data_ptr()), 8, p(c.data_ptr()), L, 1,
                                  95, 80, 5e-6, 1.0, p(out.data_ptr()), None)
    assert st == 6 and "whole" in N.last_error()
