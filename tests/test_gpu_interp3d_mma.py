"""The 3-D tensor-core interp (k_interp3d_mma: on the spread's 4 x 8 x 16 tiles, per tile a
TF32 GEMM of the tile's samples' (y, z) weights against the tile's grid values, the x planes
contracted per sample, partial sums over a sample's tiles added with float atomics) against
the FP64 oracle and against the plane-streaming interp.

Covered: coil counts that fill one group of 8 and that leave a partial second group, split
tiles (interleaved work items), odd oversampled grids with partial edge tiles, output
weights, coil-last and coil-major (strided) sample layouts, few samples (mostly empty
tiles), multiple trajectory groups, the type-2 and type-21 drivers, and the status word.

Tolerance: TOL_REF = 2e-5 relative L2 against the FP64 oracle; 5e-6 against the FP32
plane-streaming interp (3-term TF32 products, FP32 accumulation in the tensor core).
"""
import numpy as np
import pytest
import torch

import oracle as O
from mripy_gb300.plan import NufftPlan, Tuning

pytestmark = pytest.mark.gpu

TOL_REF = 2e-5
TOL_PLANES = 5e-6


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
    xs[:, :nd] *= 0.08                                      # dense centre: split tiles
    xs[:, nd:nd + 100] = np.pi                              # stencils across the periodic edge
    return xs


def _pair(shape, nc, xs, eps=5e-6, max_subproblem=0):
    """The same plan with the tensor-core interp (default) and with the plane-streaming one."""
    out = []
    for iv in (0, 1):
        p = NufftPlan(3, shape, n_coil=nc, eps=eps, max_nspread=6,
                      tuning=Tuning(max_subproblem=max_subproblem, interp_variant=iv))
        p.set_points([cuda(v) for v in xs])
        assert p.info()["spread_tile"] == (4, 8, 16)
        out.append(p)
    return out


@pytest.mark.parametrize("nc", [8, 12, 16])
def test_interp_mma_type2_against_oracle_and_planes(nc):
    rng = np.random.default_rng(80 + nc)
    M, shape = 9000, (26, 24, 28)
    xs = _points(rng, M)
    F = cvec(rng, shape + (nc,))
    pm, pp = _pair(shape, nc, xs, max_subproblem=256)
    cm = pm.type2(cuda(F[None]))
    cp = pp.type2(cuda(F[None]))
    pm.status()
    pp.status()
    assert pm.info()["split_tiles"] > 0
    ref = O.nufft_type2(tuple(xs), F.astype(np.complex128), shape, eps=5e-6)
    assert rel(cm, ref) < TOL_REF
    assert float((cm - cp).norm() / cp.norm()) < TOL_PLANES
    pm.close()
    pp.close()


def test_interp_mma_odd_grid_weights_and_strided_output():
    """Odd oversampled grid 63 x 57 x 69 (ratio 3) with partial edge tiles; per-sample output
    weights; the same interp into a coil-major (strided) sample layout."""
    rng = np.random.default_rng(81)
    M, shape, nc = 7000, (21, 19, 23), 8
    xs = _points(rng, M)
    pm, pp = _pair(shape, nc, xs, eps=1e-12)
    assert pm.info()["nf"] == (63, 57, 69)
    g = cuda(cvec(rng, (nc,) + pm.info()["nf"]))
    w = cuda(rng.uniform(0.5, 1.5, M).astype(np.float32))
    a = pm.interp(g, weight=w)
    b = pp.interp(g, weight=w)
    assert float((a - b).norm() / b.norm()) < TOL_PLANES
    cm = torch.empty((nc, M), dtype=torch.complex64, device="cuda").t()   # coil-major: strided
    pm.interp(g, out=cm, weight=w)
    pm.status()
    assert float((cm - a).abs().max()) <= 1e-6 * float(a.abs().max())
    pm.close()
    pp.close()


def test_interp_mma_sparse_trajectory_and_groups():
    """Two trajectory groups of few samples (most tiles empty work items): every output
    sample is written (the launcher zeroes the output before the atomics)."""
    rng = np.random.default_rng(82)
    shape, nc = (32, 32, 32), 8
    xs = rng.uniform(-np.pi, np.pi, (3, 600))
    F = cvec(rng, (2,) + shape + (nc,))
    out = []
    for iv in (0, 1):
        p = NufftPlan(3, shape, n_coil=nc, n_traj=2, eps=5e-6, max_nspread=6, tuning=Tuning(interp_variant=iv))
        p.set_points([cuda(v) for v in xs], traj_offsets=[0, 250, 600])
        s = torch.full((600, nc), float("nan"), dtype=torch.complex64, device="cuda")
        p.type2(cuda(F), out=s)
        p.status()
        assert torch.isfinite(torch.view_as_real(s)).all()
        out.append(s.clone())
        p.close()
    assert float((out[0] - out[1]).norm() / out[1].norm()) < TOL_PLANES
    for gidx, (a, b) in enumerate(((0, 250), (250, 600))):
        ref = O.nufft_type2(tuple(x[a:b] for x in xs), F[gidx].astype(np.complex128), shape, eps=5e-6)
        assert rel(out[0][a:b], ref) < TOL_REF


def test_interp_mma_type21_matches_planes():
    rng = np.random.default_rng(83)
    M, shape, nc = 12000, (32, 32, 32), 8
    xs = _points(rng, M)
    F = cuda(cvec(rng, (1,) + shape + (nc,)))
    dcf = cuda(rng.uniform(0.5, 1.5, M).astype(np.float32))
    pm, pp = _pair(shape, nc, xs)
    a = pm.type21(F, dcf=dcf)
    b = pp.type21(F, dcf=dcf)
    pm.status()
    assert float((a - b).norm() / b.norm()) < TOL_PLANES
    pm.close()
    pp.close()
