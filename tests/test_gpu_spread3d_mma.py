"""The 3-D tensor-core spread (k_spread_mma<3, ...>: per 4 x 8 x 16 tile a TF32 GEMM over the
tile's samples, operands split into hi + lo parts, A built in TMEM, B in swizzled shared
memory, the accumulator in TMEM) against the FP64 oracle.

Covered: coil counts that fill one group of 8 and that leave a partial second group (also
with dense tiles), split tiles (global-atomic flush), dense tiles (the compensated instance:
the batches' accumulators summed in FP32 groups folded into Kahan sums; its centre-cell
error against FP64 on 3-D radial data), long work items (many passes over the batch ring and
both operand buffers), stencils across the periodic edge, odd oversampled grids with partial
edge tiles, a grid buffer that is not 16-byte aligned, density weights, empty work items
(zeros written without an MMA), ragged trajectory groups, run-to-run bit equality, agreement
with the FP32 cube kernel, and the status word (clean after every call).

Tolerance: TOL_REF = 2e-5 relative L2 against the FP64 oracle (the 3-term TF32 products are
within ~1e-6 of FP32); 5e-6 relative L2 against the FP32 cube kernel.
"""
import numpy as np
import pytest
import torch

import oracle as O
from mripy_gb300.plan import NufftPlan, Tuning

pytestmark = pytest.mark.gpu

TOL_REF = 2e-5
TOL_CUBE = 5e-6
MMA = Tuning(coil_group=8, spread_variant=3)


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def cvec(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def rel(a, b):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _points(rng, M, dense=0.4):
    xs = rng.uniform(-np.pi, np.pi, (3, M))
    nd = int(M * dense)
    xs[:, :nd] *= 0.08                                      # dense centre: split and dense tiles
    xs[:, nd:nd + 100] = np.pi                              # stencils across the periodic edge
    return xs


def _plan(shape, nc, xs, tuning=MMA, **kw):
    p = NufftPlan(3, shape, n_coil=nc, eps=kw.pop("eps", 5e-6), max_nspread=6, tuning=tuning, **kw)
    p.set_points([cuda(v) for v in xs])
    assert p.info()["spread_tile"] == (4, 8, 16)
    return p


@pytest.mark.parametrize("nc", [8, 12, 16])
def test_mma_against_oracle(nc):
    rng = np.random.default_rng(70 + nc)
    M, shape = 9000, (26, 24, 28)
    xs = _points(rng, M)
    p = _plan(shape, nc, xs, tuning=Tuning(coil_group=8, spread_variant=3, max_subproblem=256))
    c = cvec(rng, (M, nc))
    w = rng.uniform(0.5, 1.5, M)
    F = p.type1(cuda(c), weight=cuda(w.astype(np.float32)))
    p.status()
    Fo = O.nufft_type1(tuple(xs), (c * w[:, None]).astype(np.complex128), shape, eps=5e-6)
    assert rel(F[0], Fo) < TOL_REF
    p.close()


@pytest.mark.parametrize("dense_tile_samples,max_subproblem", [(0, 64), (200, 256), (200, 4096), (-1, 4096)])
def test_mma_split_dense_and_long_items(dense_tile_samples, max_subproblem):
    """Many split tiles (64-sample items), dense tiles on the compensated instance (low
    threshold), and long items that reuse every ring slot and operand buffer many times."""
    rng = np.random.default_rng(71)
    M, shape, nc = 20000, (24, 24, 24), 8
    xs = _points(rng, M, dense=0.6)
    p = _plan(shape, nc, xs, tuning=Tuning(coil_group=8, spread_variant=3, max_subproblem=max_subproblem),
              dense_tile_samples=dense_tile_samples)
    inf = p.info()
    if dense_tile_samples > 0:
        assert inf["dense_subproblems"] > 0
    if max_subproblem == 64:
        assert inf["split_tiles"] > 0
    c = cvec(rng, (M, nc))
    F = p.type1(cuda(c))
    p.status()
    assert rel(F[0], O.nufft_type1(tuple(xs), c.astype(np.complex128), shape, eps=5e-6)) < TOL_REF
    p.close()


@pytest.mark.parametrize("nc", [12, 16])
def test_mma_dense_tiles_with_two_coil_groups(nc):
    """Dense tiles (low threshold) with two coil groups: the compensated instance runs one
    block per (dense subproblem, coil group) through the plan's list of dense subproblems."""
    rng = np.random.default_rng(76 + nc)
    M, shape = 15000, (24, 24, 24)
    xs = _points(rng, M, dense=0.6)
    p = _plan(shape, nc, xs, tuning=Tuning(coil_group=8, spread_variant=3, max_subproblem=512),
              dense_tile_samples=300)
    assert p.info()["dense_subproblems"] > 0
    c = cvec(rng, (M, nc))
    F = p.type1(cuda(c))
    p.status()
    assert rel(F[0], O.nufft_type1(tuple(xs), c.astype(np.complex128), shape, eps=5e-6)) < TOL_REF
    p.close()


def test_mma_odd_grid_edge_tiles_and_unaligned_buffer():
    """Ratio 3 (eps 1e-12, nspread clamped to 6): odd oversampled grid 63 x 57 x 69, partial
    tiles at the upper edges; then the same spread into a grid buffer that starts 8 bytes
    past a 16-byte boundary."""
    rng = np.random.default_rng(72)
    M, shape, nc = 7000, (21, 19, 23), 8
    xs = _points(rng, M)
    p = _plan(shape, nc, xs, eps=1e-12)
    assert p.info()["nf"] == (63, 57, 69)
    c = cvec(rng, (M, nc))
    Fo = O.nufft_type1(tuple(xs), c.astype(np.complex128), shape, eps=1e-12)
    assert rel(p.type1(cuda(c))[0], Fo) < TOL_REF
    dc = cuda(c)
    ref = p.spread(dc, grid=p.grid()).clone()
    buf = torch.empty(ref.numel() + 1, dtype=torch.complex64, device="cuda")
    view = buf[1:].view(ref.shape)
    assert view.data_ptr() % 16 == 8
    p.spread(dc, grid=view)
    p.status()
    assert float((view - ref).abs().max()) <= 1e-6 * float(ref.abs().max())
    p.close()


def test_mma_sparse_trajectory_with_empty_tiles():
    """Few samples: most tiles are empty work items, written as zeros without an MMA."""
    rng = np.random.default_rng(74)
    M, shape, nc = 300, (32, 32, 32), 8
    xs = rng.uniform(-np.pi, np.pi, (3, M))
    p = _plan(shape, nc, xs)
    c = cvec(rng, (M, nc))
    p.grid().fill_(float("nan"))
    F = p.type1(cuda(c))
    p.status()
    assert torch.isfinite(torch.view_as_real(F)).all()
    assert rel(F[0], O.nufft_type1(tuple(xs), c.astype(np.complex128), shape, eps=5e-6)) < TOL_REF
    p.close()


def test_mma_bitwise_repeatable_and_close_to_cube_kernel():
    """Without split tiles two spreads are bit-equal; the tensor-core and FP32 cube kernels
    on the same tile agree to the 3-term TF32 products' rounding."""
    rng = np.random.default_rng(73)
    M, shape, nc = 12000, (32, 32, 32), 8
    xs = _points(rng, M)
    c = cuda(cvec(rng, (M, nc)))
    out = {}
    for var in (2, 3):
        tu = Tuning(spread_tile=(4, 8, 16), coil_group=8, spread_variant=var, max_subproblem=1 << 20)
        p = NufftPlan(3, shape, n_coil=nc, eps=5e-6, max_nspread=6, tuning=tu, dense_tile_samples=-1)
        p.set_points([cuda(v) for v in xs])
        assert p.info()["split_tiles"] == 0
        a = p.spread(c, grid=p.grid()).clone()
        b = p.spread(c, grid=p.grid()).clone()
        p.status()
        assert torch.equal(a, b)
        out[var] = a
        p.close()
    assert float((out[3] - out[2]).norm() / out[2].norm()) < TOL_CUBE


def test_mma_compensated_centre_tiles_3d_radial():
    """Dense k-space-centre tiles of 3-D centre-out radial data (8 coils) run the compensated
    tensor-core instance: every batch's accumulator is drained into an FP32 group sum that is
    folded every 8 batches into a Kahan-compensated FP32 sum.  Against the FP64 oracle spread
    the centre cells' error drops (measured on GB300: 1.7e-6 uncompensated -> 3.8e-7; the FP32
    cube kernel: 7.5e-7 -> 1.3e-7)."""
    from mripy_gb300 import synth
    rng = np.random.default_rng(30)
    n, nc = 32, 8
    xs = [2 * np.pi * k for k in synth.centre_out_radial_3d(4000, 32)]
    M = len(xs[0])
    c = rng.standard_normal((M, nc)) + 1j * rng.standard_normal((M, nc))
    ns, nf, tau = O.grid_params(3, n, n, n, eps=5e-6, max_nspread=6)
    ref = O.spread(xs, c.T, tau, ns, nf)
    centre = np.abs(ref) > np.percentile(np.abs(ref), 99.9)
    errs = {}
    for dense in (2048, -1):
        p = NufftPlan(3, (n, n, n), n_coil=nc, eps=5e-6, max_nspread=6, dense_tile_samples=dense,
                      tuning=Tuning(max_subproblem=4096)).set_points([cuda(v) for v in xs])
        assert p.info()["spread_tile"] == (4, 8, 16)
        assert (p.info()["dense_subproblems"] > 0) == (dense > 0)
        g = p.spread(cuda(c.astype(np.complex64))).cpu().numpy()
        p.status()
        errs[dense] = np.linalg.norm((g - ref)[centre]) / np.linalg.norm(ref[centre])
        p.close()
    assert errs[2048] < 6e-7
    assert errs[2048] < 0.4 * errs[-1]


def test_mma_ragged_trajectory_groups():
    """Three trajectory groups of unequal size (one of 30 samples) in one plan: each group's
    grid against the oracle, through the work items' group index."""
    rng = np.random.default_rng(75)
    shape, nc = (28, 28, 28), 8
    counts = [6000, 30, 4000]
    off = np.concatenate([[0], np.cumsum(counts)])
    xs = _points(rng, int(off[-1]))
    c = cvec(rng, (int(off[-1]), nc))
    p = NufftPlan(3, shape, n_coil=nc, n_traj=3, eps=5e-6, max_nspread=6, tuning=MMA)
    p.set_points([cuda(v) for v in xs], traj_offsets=[int(v) for v in off])
    assert p.info()["spread_tile"] == (4, 8, 16)
    F = p.type1(cuda(c))
    p.status()
    for k in range(3):
        a, b = int(off[k]), int(off[k + 1])
        Fo = O.nufft_type1(tuple(x[a:b] for x in xs), c[a:b].astype(np.complex128), shape, eps=5e-6)
        assert rel(F[k], Fo) < TOL_REF
    p.close()
