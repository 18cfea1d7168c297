"""The 3-D cube spread kernel (k_spread3d_cube: 4^3-cell register cubes per consumer warp,
producer warps feeding a ring of sample batches on mbarriers, persistent blocks) against
the FP64 oracle.

Covered: every tile shape it takes (8 and 16 cubes), coil counts that fill one group of 8
and that leave a partial second group, split tiles (global-atomic flush), the Kahan-
compensated instance for dense tiles, stencils across the periodic edge, odd oversampled
grids and partial edge tiles (scalar stores), a grid buffer that is not 16-byte aligned
(scalar stores), density weights, long work items (many passes over the ring), empty
tiles, and the ring's status bit (clean after every call).

Tolerance: TOL_REF = 2e-5 relative L2 (FP32 accumulation against the FP64 oracle).
"""
import numpy as np
import pytest
import torch

import oracle as O
from mripy_gb300.plan import NufftPlan, Tuning

pytestmark = pytest.mark.gpu

TOL_REF = 2e-5


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


@pytest.mark.parametrize("tile", [(8, 8, 8), (4, 8, 16), (8, 8, 16), (16, 8, 8), (8, 16, 8), (4, 16, 16)])
@pytest.mark.parametrize("nc", [8, 12])
def test_cube_tiles_against_oracle(tile, nc):
    rng = np.random.default_rng(60 + nc)
    M, shape = 9000, (26, 24, 28)
    xs = _points(rng, M)
    tu = Tuning(spread_tile=tile, coil_group=8, spread_variant=2, max_subproblem=256)
    p = NufftPlan(3, shape, n_coil=nc, eps=5e-6, max_nspread=6, tuning=tu).set_points([cuda(v) for v in xs])
    c = cvec(rng, (M, nc))
    w = rng.uniform(0.5, 1.5, M)
    F = p.type1(cuda(c), weight=cuda(w.astype(np.float32)))
    p.status()
    Fo = O.nufft_type1(tuple(xs), (c * w[:, None]).astype(np.complex128), shape, eps=5e-6)
    assert rel(F[0], Fo) < TOL_REF
    p.close()


@pytest.mark.parametrize("dense_tile_samples,max_subproblem", [(0, 64), (200, 256), (200, 4096), (-1, 4096)])
def test_cube_split_dense_and_long_items(dense_tile_samples, max_subproblem):
    """Many split tiles (64-sample items), the compensated instance on dense tiles (low
    threshold), and long items that pass over every ring slot many times."""
    rng = np.random.default_rng(61)
    M, shape, nc = 20000, (24, 24, 24), 8
    xs = _points(rng, M, dense=0.6)
    tu = Tuning(spread_tile=(8, 8, 8), coil_group=8, spread_variant=2, max_subproblem=max_subproblem)
    p = NufftPlan(3, shape, n_coil=nc, eps=5e-6, max_nspread=6, tuning=tu,
                  dense_tile_samples=dense_tile_samples).set_points([cuda(v) for v in xs])
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


def test_cube_odd_grid_edge_tiles_and_unaligned_buffer():
    """Ratio 3 (eps 1e-12, nspread clamped to 6): odd oversampled grid 63 x 57 x 69, partial
    tiles at the upper edges, scalar stores; then the same spread into a grid buffer that
    starts 8 bytes past a 16-byte boundary."""
    rng = np.random.default_rng(62)
    M, shape, nc = 7000, (21, 19, 23), 8
    xs = _points(rng, M)
    tu = Tuning(spread_tile=(8, 8, 16), coil_group=8, spread_variant=2)
    p = NufftPlan(3, shape, n_coil=nc, eps=1e-12, max_nspread=6, tuning=tu).set_points([cuda(v) for v in xs])
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


def test_cube_sparse_trajectory_with_empty_tiles():
    """Few samples: most tiles are empty work items, written as zeros by the cube kernel."""
    rng = np.random.default_rng(64)
    M, shape, nc = 300, (32, 32, 32), 8
    xs = rng.uniform(-np.pi, np.pi, (3, M))
    tu = Tuning(spread_tile=(8, 8, 8), coil_group=8, spread_variant=2)
    p = NufftPlan(3, shape, n_coil=nc, eps=5e-6, max_nspread=6, tuning=tu).set_points([cuda(v) for v in xs])
    c = cvec(rng, (M, nc))
    g = p.grid()
    g.fill_(float("nan"))
    F = p.type1(cuda(c))
    p.status()
    assert torch.isfinite(torch.view_as_real(F)).all()
    assert rel(F[0], O.nufft_type1(tuple(xs), c.astype(np.complex128), shape, eps=5e-6)) < TOL_REF
    p.close()


def test_cube_matches_warp_rows_kernel():
    """The cube kernel and the warp-row register kernel on the same tile agree to rounding."""
    rng = np.random.default_rng(63)
    M, shape, nc = 12000, (32, 32, 32), 8
    xs = _points(rng, M)
    c = cuda(cvec(rng, (M, nc)))
    out = []
    for var in (1, 2):
        tu = Tuning(spread_tile=(4, 8, 16), coil_group=8, threads=256, spread_variant=var)
        p = NufftPlan(3, shape, n_coil=nc, eps=5e-6, max_nspread=6, tuning=tu).set_points([cuda(v) for v in xs])
        out.append(p.spread(c, grid=p.grid()).clone())
        p.status()
        p.close()
    assert float((out[0] - out[1]).norm() / out[1].norm()) < 1e-6
