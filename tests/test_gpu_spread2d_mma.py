"""The 2-D tensor-core spread (k_spread_mma<2, ...>: per 8 x 16 tile a TF32 GEMM over the tile's
samples, A = wx (x) wy in TMEM, B = the coil values in swizzled shared memory, N = 8 coils x
re/im; `spread_variant` 3) against the FP64 oracle and the FP32 register kernel.

Covered: coil counts that fill one group of 8 and that leave a partial second group, split
tiles (interleaved work items, global-atomic flush), long work items (group drains), odd
oversampled grids with partial edge tiles, a grid buffer that is not 16-byte aligned,
density weights, ragged trajectory groups, mostly empty tiles, run-to-run bit equality
without split tiles, and the status word.

Tolerance: TOL_REF = 2e-5 relative L2 against the FP64 oracle; 5e-6 against the FP32
register kernel.
"""
import numpy as np
import pytest
import torch

import oracle as O
from mripy_gb300.plan import NufftPlan, Tuning

pytestmark = pytest.mark.gpu

TOL_REF = 2e-5
TOL_FP32 = 5e-6


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def cvec(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def rel(a, b):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _points(rng, M, dense=0.4):
    xs = rng.uniform(-np.pi, np.pi, (2, M))
    nd = int(M * dense)
    xs[:, :nd] *= 0.08                                      # dense centre: split tiles
    xs[:, nd:nd + 100] = np.pi                              # stencils across the periodic edge
    return xs


def _plan(shape, nc, xs, max_subproblem=0, variant=3, eps=5e-6, n_traj=1, offsets=None, max_nspread=None):
    p = NufftPlan(2, shape, n_coil=nc, n_traj=n_traj, eps=eps, max_nspread=max_nspread,
                  tuning=Tuning(spread_variant=variant, max_subproblem=max_subproblem))
    p.set_points([cuda(v) for v in xs], traj_offsets=offsets)
    if variant == 3:
        assert p.info()["spread_tile"] == (8, 16) and p.info()["spread_variant"] == 3
    return p


@pytest.mark.parametrize("nc,max_subproblem", [(8, 64), (12, 256), (16, 0)])
def test_mma2d_against_oracle_and_register_kernel(nc, max_subproblem):
    rng = np.random.default_rng(90 + nc)
    M, shape = 20000, (60, 52)
    xs = _points(rng, M)
    c = cvec(rng, (M, nc))
    w = rng.uniform(0.5, 1.5, M)
    pm = _plan(shape, nc, xs, max_subproblem)
    pr = _plan(shape, nc, xs, variant=0)
    if max_subproblem == 64:
        assert pm.info()["split_tiles"] > 0
    F = pm.type1(cuda(c), weight=cuda(w.astype(np.float32)))
    Fr = pr.type1(cuda(c), weight=cuda(w.astype(np.float32)))
    pm.status()
    Fo = O.nufft_type1(tuple(xs), (c * w[:, None]).astype(np.complex128), shape, eps=5e-6)
    assert rel(F[0], Fo) < TOL_REF
    assert float((F - Fr).norm() / Fr.norm()) < TOL_FP32
    pm.close()
    pr.close()


def test_mma2d_odd_grid_edge_tiles_and_unaligned_buffer():
    """Ratio 3 (eps 1e-12, nspread clamped to 6): odd oversampled grid, partial tiles at the
    upper edges, against the register kernel on the same grid; then the same spread into a
    grid buffer 8 bytes past a 16-byte boundary."""
    rng = np.random.default_rng(91)
    M, shape, nc = 9000, (41, 37), 8
    xs = _points(rng, M)
    p = _plan(shape, nc, xs, eps=1e-12, max_nspread=6)
    pr = _plan(shape, nc, xs, eps=1e-12, max_nspread=6, variant=0)
    assert p.info()["nf"] == (123, 111)
    c = cvec(rng, (M, nc))
    dc = cuda(c)
    F, Fr = p.type1(dc), pr.type1(dc)
    assert float((F - Fr).norm() / Fr.norm()) < TOL_FP32
    pr.close()
    ref = p.spread(dc, grid=p.grid()).clone()
    buf = torch.empty(ref.numel() + 1, dtype=torch.complex64, device="cuda")
    view = buf[1:].view(ref.shape)
    assert view.data_ptr() % 16 == 8
    p.spread(dc, grid=view)
    p.status()
    assert float((view - ref).abs().max()) <= 1e-6 * float(ref.abs().max())
    p.close()


def test_mma2d_ragged_groups_and_empty_tiles():
    """Three trajectory groups of unequal size (one with 40 samples: most of its tiles are
    empty work items, written as zeros without an MMA)."""
    rng = np.random.default_rng(92)
    shape, nc = (64, 64), 8
    counts = [9000, 40, 5000]
    off = np.concatenate([[0], np.cumsum(counts)])
    xs = _points(rng, int(off[-1]))
    c = cvec(rng, (int(off[-1]), nc))
    p = _plan(shape, nc, xs, n_traj=3, offsets=[int(v) for v in off])
    g = p.grid()
    g.fill_(float("nan"))
    F = p.type1(cuda(c))
    p.status()
    assert torch.isfinite(torch.view_as_real(F)).all()
    for k in range(3):
        a, b = int(off[k]), int(off[k + 1])
        Fo = O.nufft_type1(tuple(x[a:b] for x in xs), c[a:b].astype(np.complex128), shape, eps=5e-6)
        assert rel(F[k], Fo) < TOL_REF
    p.close()


def test_mma2d_bitwise_repeatable_without_split_tiles():
    rng = np.random.default_rng(93)
    M, shape, nc = 30000, (64, 48), 8
    xs = _points(rng, M)
    p = _plan(shape, nc, xs, max_subproblem=1 << 20)
    assert p.info()["split_tiles"] == 0
    c = cuda(cvec(rng, (M, nc)))
    a = p.spread(c, grid=p.grid()).clone()
    b = p.spread(c, grid=p.grid()).clone()
    p.status()
    assert torch.equal(a, b)
    p.close()
