"""GPU parity: the sm_103a NUFFT against mripy's own outputs (golden vectors), the FP64
oracle restatement, and the exact NUDFT.

Tolerances (relative L2):
  TOL_REF = 2e-5  GPU (complex64 data, FP32 stencil) vs the reference / oracle at the
                  same eps (FP64): the difference is FP32 rounding only
  TOL_EXACT = 1e-4  vs the FP64 NUDFT at nspread 6 (the accuracy target)
"""
import os

import numpy as np
import pytest
import torch

import oracle as O
from mripy_gb300 import nufft_func as nf
from mripy_gb300 import operators as ops
from mripy_gb300 import synth
from mripy_gb300._native import GbnError
from mripy_gb300.plan import NufftPlan, Tuning

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden")
TOL_REF = 2e-5
TOL_EXACT = 1e-4


def rel(a, b):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def cvec(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


# ------------------------------------------------------------------ golden vectors
@pytest.fixture(scope="module")
def g1():
    return np.load(os.path.join(G, "golden_1d.npz"))


@pytest.fixture(scope="module")
def g2():
    return np.load(os.path.join(G, "golden_2d.npz"))


@pytest.fixture(scope="module")
def g3():
    return np.load(os.path.join(G, "golden_3d.npz"))


@pytest.mark.parametrize("eps,tag", [(5e-6, "e5em6"), (1e-3, "e1em3")])
@pytest.mark.parametrize("df", [1.0, 2.0])
@pytest.mark.parametrize("iflag", [1, -1])
def test_golden_1d(g1, eps, tag, df, iflag):
    key = "%s_df%d_if%+d" % (tag, int(df), iflag)
    x, c, Fk = g1["x"], g1["c"], g1["Fk"]
    assert rel(nf.nufft1d1_gaussker(x, c, 20, df=df, eps=eps, iflag=iflag), g1["t1_" + key]) < TOL_REF
    assert rel(nf.nufft1d2_gaussker(x, Fk, 20, df=df, eps=eps, iflag=iflag), g1["t2_" + key]) < TOL_REF
    assert rel(nf.nufft1d21_gaussker(x, Fk, 20, df=df, eps=eps, iflag=iflag), g1["t21_" + key]) < TOL_REF


@pytest.mark.parametrize("eps,tag", [(5e-6, "e5em6"), (1e-5, "e1em5")])
@pytest.mark.parametrize("df", [1.0, 2.0])
@pytest.mark.parametrize("iflag", [1, -1])
def test_golden_2d(g2, eps, tag, df, iflag):
    key = "a_%s_df%d_if%+d" % (tag, int(df), iflag)
    x, y, c, Fk = g2["a_x"], g2["a_y"], g2["a_c"], g2["a_Fk"]
    out1 = nf.nufft2d1_gaussker(x, y, c, 16, 16, df=df, eps=eps, iflag=iflag)
    assert out1.dtype == np.complex128 and out1.shape == (16, 16)
    assert rel(out1, g2["t1_" + key]) < TOL_REF
    assert rel(nf.nufft2d2_gaussker(x, y, Fk, 16, 16, df=df, eps=eps, iflag=iflag), g2["t2_" + key]) < TOL_REF
    assert rel(nf.nufft2d21_gaussker(x, y, Fk, 16, 16, df=df, eps=eps, iflag=iflag), g2["t21_" + key]) < TOL_REF


@pytest.mark.parametrize("eps,tag", [(1e-5, "e1em5"), (1e-3, "e1em3")])
def test_golden_2d_coils_odd_sizes(g2, eps, tag):
    key = "b_" + tag
    x, y, c, Fk = g2["b_x"], g2["b_y"], g2["b_c"], g2["b_Fk"]
    assert rel(nf.nufft2d1_gaussker_cuda(x, y, c, 15, 12, eps=eps), g2["t1_" + key]) < TOL_REF
    assert rel(nf.nufft2d2_gaussker_cuda(x, y, Fk, 15, 12, eps=eps), g2["t2_" + key]) < TOL_REF
    assert rel(nf.nufft2d21_gaussker_cuda(x, y, Fk, 15, 12, eps=eps), g2["t21_" + key]) < TOL_REF


@pytest.mark.parametrize("eps,tag", [(5e-6, "e5em6"), (1e-5, "e1em5")])
@pytest.mark.parametrize("iflag", [1, -1])
def test_golden_3d(g3, eps, tag, iflag):
    key = "a_%s_if%+d" % (tag, iflag)
    x, y, z, c, Fk, dcf = (g3[k] for k in ("a_x", "a_y", "a_z", "a_c", "a_Fk", "a_dcf"))
    assert rel(nf.nufft3d1_gaussker(x, y, z, c, 8, 8, 6, eps=eps, iflag=iflag), g3["t1_" + key]) < TOL_REF
    assert rel(nf.nufft3d2_gaussker(x, y, z, Fk, 8, 8, 6, eps=eps, iflag=iflag), g3["t2_" + key]) < TOL_REF
    assert rel(nf.nufft3d21_gaussker(x, y, z, Fk, 8, 8, 6, dcf=dcf, eps=eps, iflag=iflag),
               g3["t21_" + key]) < TOL_REF


def test_golden_3d_clamp_and_cuda_names(g3):
    x, y, z, c = (g3[k] for k in ("a_x", "a_y", "a_z", "a_c"))
    assert rel(nf.nufft3d1_gaussker_cuda(x, y, z, c, 8, 8, 6, eps=1e-12), g3["t1_a_e1em12_if+1"]) < TOL_REF


def test_golden_operator_nufft3d(g3):
    for cls in (ops.NUFFT3d, ops.NUFFT3d_cuda):
        op = cls(tuple(int(v) for v in g3["b_shape"]), g3["b_dcf"])
        op.normalize_set_ktraj(g3["b_ktraj"].copy())
        assert rel(op.forward(g3["b_im"]), g3["b_forward"]) < TOL_REF
        assert rel(op.backward(g3["b_kdata"]), g3["b_backward"]) < TOL_REF
        assert rel(op.forward_backward(g3["b_im"]), g3["b_forward_backward"]) < TOL_REF


# ------------------------------------------------------------------ configuration 1 at full size
def test_config1_against_oracle_and_nudft():
    cfg = synth.config1()
    kx, ky = cfg["k"]
    x, y = 2 * np.pi * kx, 2 * np.pi * ky
    img = cfg["image"]
    # forward (type-2) and adjoint (type-1), drop-in functions, nspread 6
    c_gpu = nf.nufft2d2_gaussker(x, y, img, 128, 128, eps=5e-6)
    c_orc = O.nufft_type2((x, y), img.astype(np.complex128), (128, 128), eps=5e-6)
    assert rel(c_gpu, c_orc) < TOL_REF
    rng = np.random.default_rng(7)
    sub = rng.choice(len(x), 4096, replace=False)
    c_exact = O.nudft_type2((x[sub], y[sub]), img.astype(np.complex128), (128, 128))
    assert rel(c_gpu[sub], c_exact) < TOL_EXACT

    cdat = cvec(rng, len(x)).astype(np.complex128)
    F_gpu = nf.nufft2d1_gaussker(x, y, cdat, 128, 128, eps=5e-6)
    F_orc = O.nufft_type1((x, y), cdat, (128, 128), eps=5e-6)
    assert rel(F_gpu, F_orc) < TOL_REF
    pix = rng.choice(128 * 128, 1024, replace=False)
    F_exact = O.nudft_type1((x, y), cdat, (128, 128), pixels=pix)
    assert rel(F_gpu.reshape(-1)[pix], F_exact) < TOL_EXACT


def test_adjoint_identity_plan():
    rng = np.random.default_rng(11)
    M = 20000
    x = cuda(rng.uniform(-np.pi, np.pi, M))
    y = cuda(rng.uniform(-np.pi, np.pi, M))
    p = NufftPlan(2, (96, 80), n_coil=2, eps=5e-6).set_points([x, y])
    F = cuda(cvec(rng, (1, 96, 80, 2)))
    c = cuda(cvec(rng, (M, 2)))
    AF = p.type2(F)
    ATc = p.type1(c) * M            # type-1 carries 1/M
    lhs = torch.vdot(c.reshape(-1), AF.reshape(-1)).item()
    rhs = torch.vdot(ATc.reshape(-1), F.reshape(-1)).item()
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


# ------------------------------------------------------------------ layouts, coils, ragged groups
def test_coil_layouts_and_oracle():
    rng = np.random.default_rng(12)
    M, nc = 5000, 3
    xs = rng.uniform(-3 * np.pi, 3 * np.pi, (2, M))           # wraps mod 2 pi
    p = NufftPlan(2, (40, 36), n_coil=nc, eps=1e-5).set_points([cuda(xs[0]), cuda(xs[1])])
    c_np = cvec(rng, (M, nc))
    c_last = cuda(c_np)                                       # (M, nc) coil-last
    c_major = cuda(np.ascontiguousarray(c_np.T)).t()          # (M, nc) view of (nc, M)
    F1 = p.type1(c_last)
    F2 = p.type1(c_major)
    assert rel(F1, F2) < 1e-6
    F_orc = O.nufft_type1((xs[0], xs[1]), c_np.astype(np.complex128), (40, 36), eps=1e-5)
    assert rel(F1[0], F_orc) < TOL_REF
    img = cvec(rng, (40, 36, nc))
    k1 = p.type2(cuda(img)[None])
    img_major = cuda(np.ascontiguousarray(np.moveaxis(img, -1, 0)))   # (nc, 40, 36)
    k2 = p.type2(img_major.permute(1, 2, 0)[None])
    assert rel(k1, k2) < 1e-6
    assert rel(k1, O.nufft_type2((xs[0], xs[1]), img.astype(np.complex128), (40, 36), eps=1e-5)) < TOL_REF


def test_ragged_groups_match_per_group_oracle():
    rng = np.random.default_rng(13)
    counts = [3000, 0, 1234, 7000]
    off = np.concatenate([[0], np.cumsum(counts)])
    M, nc = int(off[-1]), 2
    xs = rng.uniform(-np.pi, np.pi, (2, M))
    p = NufftPlan(2, (48, 48), n_coil=nc, n_traj=len(counts), eps=5e-6)
    p.set_points([cuda(xs[0]), cuda(xs[1])], traj_offsets=off.tolist())
    c = cvec(rng, (M, nc))
    F = p.type1(cuda(c)).cpu().numpy()                       # (4, 48, 48, nc)
    img = cvec(rng, (len(counts), 48, 48, nc))
    k = p.type2(cuda(img)).cpu().numpy()
    for g, (a, b) in enumerate(zip(off[:-1], off[1:])):
        if b == a:
            assert np.abs(F[g]).max() == 0.0
            continue
        Fo = O.nufft_type1((xs[0][a:b], xs[1][a:b]), c[a:b].astype(np.complex128), (48, 48), eps=5e-6)
        assert rel(F[g], Fo) < TOL_REF
        ko = O.nufft_type2((xs[0][a:b], xs[1][a:b]), img[g].astype(np.complex128), (48, 48), eps=5e-6)
        assert rel(k[a:b], ko) < TOL_REF


def test_float32_coordinates():
    rng = np.random.default_rng(14)
    xs = rng.uniform(-np.pi, np.pi, (2, 4000)).astype(np.float32)
    img = cvec(rng, (32, 32))
    out = nf.nufft2d2_gaussker(cuda(xs[0]), cuda(xs[1]), cuda(img), 32, 32, eps=1e-5)
    assert out.dtype == torch.complex64 and out.is_cuda
    ref = O.nufft_type2((xs[0].astype(np.float64), xs[1].astype(np.float64)), img.astype(np.complex128),
                        (32, 32), eps=1e-5)
    assert rel(out, ref) < TOL_REF


def test_large_nspread_generic_kernel():
    # function default eps 1e-15: ratio 3, nspread 14 (28 taps per dim, generic kernel)
    rng = np.random.default_rng(15)
    x, y = rng.uniform(-np.pi, np.pi, (2, 600))
    c = cvec(rng, 600).astype(np.complex128)
    F = cvec(rng, (20, 18)).astype(np.complex128)
    assert rel(nf.nufft2d1_gaussker(x, y, c, 20, 18), O.nufft_type1((x, y), c, (20, 18))) < TOL_REF
    assert rel(nf.nufft2d2_gaussker(x, y, F, 20, 18), O.nufft_type2((x, y), F, (20, 18))) < TOL_REF
    assert rel(nf.nufft2d1_gaussker(x, y, c, 20, 18), O.nudft_type1((x, y), c, (20, 18))) < 1e-5


def test_3d_multicoil_against_oracle():
    rng = np.random.default_rng(16)
    M, nc = 3000, 3
    xs = rng.uniform(-np.pi, np.pi, (3, M))
    c = cvec(rng, (M, nc)).astype(np.complex128)
    F = cvec(rng, (20, 18, 16, nc)).astype(np.complex128)
    dcf = rng.uniform(0.5, 1.5, M)
    for eps in (5e-6, 1e-5):
        assert rel(nf.nufft3d1_gaussker(*xs, c, 20, 18, 16, eps=eps),
                   O.nufft_type1(tuple(xs), c, (20, 18, 16), eps=eps)) < TOL_REF
        assert rel(nf.nufft3d2_gaussker(*xs, F, 20, 18, 16, eps=eps),
                   O.nufft_type2(tuple(xs), F, (20, 18, 16), eps=eps)) < TOL_REF
        assert rel(nf.nufft3d21_gaussker(*xs, F, 20, 18, 16, dcf=dcf, eps=eps),
                   O.nufft_type21(tuple(xs), F, (20, 18, 16), dcf=dcf, eps=eps)) < TOL_REF


@pytest.mark.parametrize("eps", [5e-6, 1e-5])
def test_3d_warp_kernels_against_oracle(eps):
    # grid 48x44x52 >= tile + stencil in every dimension: the warp-level 3-D spread runs;
    # 5 coils exercise a partly filled coil group
    rng = np.random.default_rng(21)
    M, nc, shape = 4000, 5, (24, 22, 26)
    xs = rng.uniform(-np.pi, np.pi, (3, M))
    xs[:, :1500] *= 0.1                                          # dense centre: split bins
    c = cvec(rng, (M, nc)).astype(np.complex128)
    F = cvec(rng, shape + (nc,)).astype(np.complex128)
    dcf = rng.uniform(0.5, 1.5, M)
    assert rel(nf.nufft3d1_gaussker(*xs, c, *shape, eps=eps), O.nufft_type1(tuple(xs), c, shape, eps=eps)) < TOL_REF
    assert rel(nf.nufft3d2_gaussker(*xs, F, *shape, eps=eps), O.nufft_type2(tuple(xs), F, shape, eps=eps)) < TOL_REF
    assert rel(nf.nufft3d21_gaussker(*xs, F, *shape, dcf=dcf, eps=eps),
               O.nufft_type21(tuple(xs), F, shape, dcf=dcf, eps=eps)) < TOL_REF


@pytest.mark.parametrize("nc,tuning", [
    (11, None),                                   # default: tensor cores on 4x8x16 tiles, coil groups of 8 and 3
    (11, Tuning(spread_variant=2)),               # cube kernel on 8^3 tiles, coil groups of 8 and 3
    (11, Tuning(spread_variant=1)),               # register rows, tile 4x8x16, coil groups of 8 and 3
    (8, Tuning(threads=128, spread_variant=1)),   # register rows, tile 4x4x16
    (4, None),                                    # register tile 4x8x32, 4 coils per block
    (8, Tuning(spread_tile=(8, 8, 32))),          # shared-memory tile kernel
    (8, Tuning(max_subproblem=64)),               # many split tiles (global-atomic flush)
])
def test_3d_spread_tiles_weights_against_oracle(nc, tuning):
    rng = np.random.default_rng(22)
    M, shape = 6000, (26, 24, 28)
    xs = rng.uniform(-np.pi, np.pi, (3, M))
    xs[:, :2500] *= 0.08                                         # dense centre
    xs[:, 2500:2600] = np.pi                                     # stencils across the periodic edge
    p = NufftPlan(3, shape, n_coil=nc, eps=5e-6, tuning=tuning).set_points([cuda(v) for v in xs])
    c = cvec(rng, (M, nc))
    w = rng.uniform(0.5, 1.5, M)
    F = p.type1(cuda(c), weight=cuda(w.astype(np.float32)))
    Fo = O.nufft_type1(tuple(xs), (c * w[:, None]).astype(np.complex128), shape, eps=5e-6)
    assert rel(F[0], Fo) < TOL_REF


# ------------------------------------------------------------------ SENSE fusion and graphs
@pytest.mark.parametrize("dim,shape,nc,eps", [
    (1, (5001,), 3, 5e-6),        # rows longer than one staged segment, coil chunks of 1
    (2, (15, 13), 3, 1e-12),      # ratio 3: odd oversampled grid 45 x 39
    (2, (1100, 1030), 2, 1e-5),   # SENSE crop: two segments per row (tau follows ms only,
                                  # so ms must be the largest size or exp(tau k^2) overflows)
    (3, (9, 7, 11), 5, 1e-12),    # odd 3-D, ratio 3
    (3, (12, 10, 8), 20, 1e-5),   # coil chunks in 3-D
])
def test_pad_crop_shapes_layouts_groups(dim, shape, nc, eps):
    rng = np.random.default_rng(23)
    counts = [700, 300]
    off = np.concatenate([[0], np.cumsum(counts)])
    M = int(off[-1])
    xs = rng.uniform(-np.pi, np.pi, (dim, M))
    # 3-D: nspread clamped to 6 as nufft3d*_gaussker does (the oracle's 3-D parameters)
    p = NufftPlan(dim, shape, n_coil=nc, n_traj=2, eps=eps, max_nspread=6 if dim == 3 else None)
    p.set_points([cuda(v) for v in xs], traj_offsets=off.tolist())
    img = cvec(rng, (2,) + shape + (nc,))
    c = cvec(rng, (M, nc))
    k_last = p.type2(cuda(img))
    img_major = cuda(np.ascontiguousarray(np.moveaxis(img, -1, 1)))          # (2, nc, *shape)
    k_major = p.type2(img_major.movedim(1, -1))
    assert rel(k_last, k_major) < 1e-6
    F = p.type1(cuda(c))
    F_major = torch.empty((2, nc) + shape, dtype=torch.complex64, device="cuda")
    p.type1(cuda(c), out=F_major.movedim(1, -1))
    assert rel(F, F_major.movedim(1, -1)) < 1e-6
    for g_, (a, b) in enumerate(zip(off[:-1], off[1:])):
        co = tuple(v[a:b] for v in xs)
        assert rel(k_last[a:b], O.nufft_type2(co, img[g_].astype(np.complex128), shape, eps=eps)) < TOL_REF
        assert rel(F[g_], O.nufft_type1(co, c[a:b].astype(np.complex128), shape, eps=eps)) < TOL_REF
    # SENSE-fused pad / crop on the same shapes against the per-coil composition
    S = cuda(cvec(rng, shape + (nc,)))
    x = cuda(cvec(rng, (2,) + shape))
    ks = p.sense_forward(x, S)
    assert rel(ks, p.type2((x[..., None] * S[None]).contiguous())) < 1e-6
    xa = p.sense_adjoint(ks, S)
    assert rel(xa, (p.type1(ks) * S.conj()[None]).sum(-1)) < 1e-5


@pytest.mark.parametrize("shape,nc,eps,tile,icg", [
    ((256, 256), 8, 5e-6, (0, 0), 0),     # 8 coils per block, default 16x16 bins
    ((192, 160), 12, 1e-5, (16, 32), 0),  # 3 groups of 4 coils, 16x32 bins
    ((96, 80), 3, 5e-6, (0, 0), 0),       # one partly filled group of 4
    ((64, 64), 2, 5e-6, (8, 16), 2),      # small grid: many windows wrap at the edge
    ((128, 96), 5, 5e-6, (0, 0), 8),      # 8-coil group with 3 empty lanes
])
def test_tma_interp_matches_thread_staging(shape, nc, eps, tile, icg):
    """The window staged by tensor copies feeds the same arithmetic in the same order as
    the thread-gathered window, so the two interp paths agree bit for bit."""
    rng = np.random.default_rng(24)
    counts = [20000, 7000]
    off = np.concatenate([[0], np.cumsum(counts)])
    M = int(off[-1])
    xs = rng.uniform(-np.pi, np.pi, (2, M))
    xs[:, :9000] *= 0.15                                        # dense centre: split bins
    plans = [NufftPlan(2, shape, n_coil=nc, n_traj=2, eps=eps,
                       tuning=Tuning(interp_tile=tile, interp_coil_group=icg, interp_staging=st))
             .set_points([cuda(xs[0]), cuda(xs[1])], traj_offsets=off.tolist()) for st in (0, 1)]
    g = plans[0].grid()
    g.copy_(torch.randn(g.shape, dtype=torch.complex64, device="cuda"))
    c_tma = plans[0].interp(g)
    c_thr = plans[1].interp(g)
    plans[0].status()                                           # no bounded wait gave up
    assert torch.equal(c_tma, c_thr)
    # and the full type-2 against the oracle for the first group
    img = cvec(rng, (2,) + shape + (nc,))
    k = plans[0].type2(cuda(img))
    plans[0].status()
    ref = O.nufft_type2((xs[0][:counts[0]], xs[1][:counts[0]]), img[0].astype(np.complex128), shape, eps=eps)
    assert rel(k[:counts[0]], ref) < TOL_REF


@pytest.mark.parametrize("nc,icg,tile", [(8, 8, (8, 8, 8)), (4, 4, (8, 4, 8)), (12, 4, (4, 8, 8))])
def test_tma_planes_3d_match_thread_staging(nc, icg, tile):
    """3-D plane-streaming interp: planes staged by tensor copies (windows inside the grid in
    y and z) and by the threads (every window) feed the same arithmetic: equal bit for bit.
    A 48^3 grid puts most 19-cell windows at an edge, so one launch mixes both paths.  (With
    8 coils the library would choose the tensor-core interp: interp_variant 1 keeps the
    plane kernel.)"""
    rng = np.random.default_rng(25)
    shape, M = (24, 24, 24), 30000
    xs = rng.uniform(-np.pi, np.pi, (3, M))
    xs[:, :12000] *= 0.2
    plans = [NufftPlan(3, shape, n_coil=nc, eps=1e-6, max_nspread=6,
                       tuning=Tuning(interp_tile=tile, interp_coil_group=icg, interp_staging=st, interp_variant=1))
             .set_points([cuda(v) for v in xs]) for st in (0, 1)]
    g = plans[0].grid()
    g.copy_(torch.randn(g.shape, dtype=torch.complex64, device="cuda"))
    c_tma = plans[0].interp(g)
    c_thr = plans[1].interp(g)
    plans[0].status()
    assert torch.equal(c_tma, c_thr)
    img = cvec(rng, (1,) + shape + (nc,))
    k = plans[0].type2(cuda(img))
    plans[0].status()
    ref = O.nufft_type2(tuple(xs), img[0].astype(np.complex128), shape, eps=1e-6)
    assert rel(k, ref) < TOL_REF


@pytest.mark.parametrize("dim", [2, 3])
def test_host_entry_points_pinned_and_pageable(dim):
    """gbn_type{1,2,21}_host give the device path's results whether the caller's arrays are
    pageable (staged copies), pinned (read and written by the kernels directly, the samples
    a spread gathers copied in bulk) or pinned at an 8-byte offset from a 16-byte boundary;
    the dcf's length is not a multiple of 16 bytes."""
    import ctypes
    from mripy_gb300 import _native as N
    rng = np.random.default_rng(25)
    shape, nc, M = ((64, 48), 4, 6001) if dim == 2 else ((20, 18, 16), 4, 5001)
    xs = rng.uniform(-np.pi, np.pi, (dim, M))
    xs[:, :2000] *= 0.1                                          # split tiles (atomic flush)
    p = NufftPlan(dim, shape, n_coil=nc, eps=5e-6, max_nspread=6 if dim == 3 else None)
    p.set_points([cuda(v) for v in xs])
    img = cvec(rng, (1,) + shape + (nc,))
    c = cvec(rng, (M, nc))
    dcf = rng.uniform(0.5, 1.5, M).astype(np.float32)
    k_dev = p.type2(cuda(img)).cpu()
    F_dev = p.type1(cuda(c)).cpu()
    N_dev = p.type21(cuda(img), dcf=cuda(dcf)).cpu()
    lib = N.lib()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    def pin_offset(t):           # pinned, starting 8 bytes past a 16-byte boundary
        flat = t.reshape(-1).view(torch.uint8)
        buf = torch.empty(flat.numel() + 8, dtype=torch.uint8).pin_memory()
        assert buf.data_ptr() % 16 == 0
        out = buf[8:].view(t.dtype).reshape(t.shape)
        out.copy_(t)
        return out

    for pinned in (False, True, "offset"):
        pin = {False: (lambda t: t), True: (lambda t: t.pin_memory()), "offset": pin_offset}[pinned]
        h_img, h_c = pin(torch.from_numpy(img)), pin(torch.from_numpy(c))
        h_dcf = pin(torch.from_numpy(dcf))
        o_k = pin(torch.empty((M, nc), dtype=torch.complex64))
        o_F = pin(torch.empty((1,) + shape + (nc,), dtype=torch.complex64))
        o_N = pin(torch.empty((1,) + shape + (nc,), dtype=torch.complex64))
        N.check(lib.gbn_type2_host(p._h, vp(h_img), vp(o_k), sp))
        N.check(lib.gbn_type1_host(p._h, vp(h_c), vp(o_F), sp))
        N.check(lib.gbn_type21_host(p._h, vp(h_img), vp(o_N), vp(h_dcf), sp))
        assert torch.equal(o_k, k_dev), pinned          # interp: fixed summation order
        assert rel(o_F, F_dev) < 1e-6, pinned           # split tiles flush with atomics
        assert rel(o_N, N_dev) < 1e-6, pinned


@pytest.mark.parametrize("dim,nc", [(2, 8), (3, 8), (2, 1)])
def test_every_tuning_candidate_matches_oracle(dim, nc):
    """Each configuration the autotuner may time (tiles, threads, coils per block, kernel
    variants they select) gives the oracle's type-2 and type-1 results."""
    from mripy_gb300 import tune
    rng = np.random.default_rng(26)
    shape, M = ((64, 56), 8000) if dim == 2 else ((28, 26, 24), 6000)
    xs = rng.uniform(-np.pi, np.pi, (dim, M))
    xs[:, :3000] *= 0.1                                          # dense centre: split tiles
    img = cvec(rng, shape + (nc,))
    c = cvec(rng, (M, nc))
    co = tuple(xs)
    ref2 = O.nufft_type2(co, img.astype(np.complex128), shape, eps=5e-6)
    ref1 = O.nufft_type1(co, c.astype(np.complex128), shape, eps=5e-6)
    coords = [cuda(v) for v in xs]
    for tu in tune.candidate_tunings(dim, nc):
        p = NufftPlan(dim, shape, n_coil=nc, eps=5e-6, max_nspread=6 if dim == 3 else None, tuning=tu)
        p.set_points(coords)
        assert rel(p.type2(cuda(img)[None]), ref2) < TOL_REF, tu
        assert rel(p.type1(cuda(c))[0], ref1) < TOL_REF, tu
        p.status()
        p.close()


def test_kahan_centre_bins_3d_radial():
    """Dense k-space-centre tiles of 3-D centre-out radial data accumulate with Kahan-
    compensated FP32 sums: against the FP64 oracle spread the centre cells' error drops
    (measured on GB300: 8.1e-7 plain -> 1.2e-7 compensated at 4096-sample work items)."""
    rng = np.random.default_rng(30)
    n, nc = 32, 4
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
        assert (p.info()["dense_subproblems"] > 0) == (dense > 0)
        g = p.spread(cuda(c.astype(np.complex64))).cpu().numpy()
        p.status()
        errs[dense] = np.linalg.norm((g - ref)[centre]) / np.linalg.norm(ref[centre])
    assert errs[2048] < 3e-7
    assert errs[2048] < 0.4 * errs[-1]


def test_sense_fused_kernels_match_composition():
    rng = np.random.default_rng(17)
    shape, nc, M = (64, 48), 4, 12000
    xs = rng.uniform(-np.pi, np.pi, (2, M))
    p = NufftPlan(2, shape, n_coil=nc, eps=5e-6).set_points([cuda(xs[0]), cuda(xs[1])])
    S = cuda(synth.coil_maps(shape, nc, rng))
    x = cuda(cvec(rng, (1,) + shape))
    dcf = cuda(rng.uniform(0.2, 1.0, M).astype(np.float32))
    k = p.sense_forward(x, S)
    k_ref = p.type2((x[..., None] * S[None]).contiguous())
    assert rel(k, k_ref) < 1e-6
    xa = p.sense_adjoint(k, S, dcf=dcf)
    xa_ref = (p.type1((k * dcf[:, None]).contiguous()) * S.conj()[None]).sum(-1)
    assert rel(xa, xa_ref) < 1e-6
    xn = p.sense_normal(x, S, dcf=dcf)
    xn_ref = (p.type21((x[..., None] * S[None]).contiguous(), dcf=dcf) * S.conj()[None]).sum(-1)
    assert rel(xn, xn_ref) < 1e-6


def test_graph_replay_matches_eager():
    rng = np.random.default_rng(18)
    shape, nc, M = (64, 64), 8, 20000
    xs = rng.uniform(-np.pi, np.pi, (2, M))
    p = NufftPlan(2, shape, n_coil=nc, eps=5e-6).set_points([cuda(xs[0]), cuda(xs[1])])
    S = cuda(synth.coil_maps(shape, nc, rng))
    xb = cuda(cvec(rng, (1,) + shape))
    ob = torch.empty_like(xb)
    eager = p.sense_normal(xb, S).clone()
    g = p.capture_normal(xb, ob, sens=S)
    g.launch()
    torch.cuda.synchronize()
    assert rel(ob, eager) < 1e-6
    xb.copy_(cuda(cvec(rng, (1,) + shape)))                  # new input, same buffer
    g.launch()
    torch.cuda.synchronize()
    assert rel(ob, p.sense_normal(xb, S)) < 1e-6
    g.close()


def test_joint_operator_fused_path_matches_generic():
    rng = np.random.default_rng(19)
    shape, nc = (48, 40), 3
    kx, ky = synth.golden_radial_2d(60, 96)
    S = synth.coil_maps(shape, nc, rng)
    nft = ops.NUFFT2d(shape)
    nft.set_ktraj(2 * np.pi * kx, 2 * np.pi * ky)
    A = ops.joint2operators(ops.espirit(S), nft)
    x = cvec(rng, shape + (1,))
    kd = A.forward(x)
    kd_ref = nft.forward(S * x)
    assert rel(kd, kd_ref) < 1e-5
    xb = A.backward(kd)
    xb_ref = np.sum(np.conj(S) * nft.backward(kd), axis=-1, keepdims=True)
    assert rel(xb, xb_ref) < 1e-5
    xn = A.forward_backward(x)
    xn_ref = np.sum(np.conj(S) * nft.forward_backward(S * x), axis=-1, keepdims=True)
    assert rel(xn, xn_ref) < 1e-5


# ------------------------------------------------------------------ trajectory gradient
def test_interp_grad_coords_against_fp64_gradients():
    rng = np.random.default_rng(20)
    shape, M = (24, 20), 300
    xs = rng.uniform(-np.pi, np.pi, (2, M))
    F = cvec(rng, shape).astype(np.complex128)
    gc = cvec(rng, M).astype(np.complex128)
    p = NufftPlan(2, shape, n_coil=1, eps=5e-6).set_points([cuda(xs[0]), cuda(xs[1])])
    grid = p.pad_deapod(cuda(F.astype(np.complex64))[None, ..., None])
    p.fft(grid, -1)
    gk = p.interp_grad_coords(grid, cuda(gc.astype(np.complex64))[:, None]).cpu().numpy()
    exact = O.nudft_type2_coord_grad((xs[0], xs[1]), F, shape, gc)
    assert rel(gk, exact) < 1e-3
    # FP64 central differences of the FP64 gridding oracle, step 1e-6
    h = 1e-6
    for j in (0, 17, 150, 299):
        for d in range(2):
            xp, xm = xs.copy(), xs.copy()
            xp[d, j] += h
            xm[d, j] -= h
            cp = O.nufft_type2((xp[0], xp[1]), F, shape, eps=5e-6)
            cm = O.nufft_type2((xm[0], xm[1]), F, shape, eps=5e-6)
            fd = np.real(np.vdot(gc, (cp - cm) / (2 * h)))
            assert abs(gk[j, d] - fd) <= 1e-3 * np.abs(exact).max()


@pytest.mark.parametrize("nc,eps", [(12, 1e-5), (3, 5e-6)])
def test_interp_grad_coords_multicoil(nc, eps):
    """The warp-per-sample 2-D gradient kernel over several coil groups (12 coils: a full
    group and a half-masked one) against the FP64 NUDFT gradient summed over the coils."""
    rng = np.random.default_rng(21)
    shape, M = (32, 28), 2500
    xs = rng.uniform(-np.pi, np.pi, (2, M))
    xs[:, :800] *= 0.2
    F = cvec(rng, shape + (nc,)).astype(np.complex128)
    gc = cvec(rng, (M, nc)).astype(np.complex128)
    p = NufftPlan(2, shape, n_coil=nc, eps=eps).set_points([cuda(xs[0]), cuda(xs[1])])
    grid = p.pad_deapod(cuda(F.astype(np.complex64))[None])
    p.fft(grid, -1)
    gk = p.interp_grad_coords(grid, cuda(gc.astype(np.complex64))).cpu().numpy()
    exact = O.nudft_type2_coord_grad((xs[0], xs[1]), F, shape, gc)            # summed over the coils
    assert rel(gk, exact) < 1e-3


# ------------------------------------------------------------------ failure paths
def test_non_finite_coordinate_is_rejected():
    x = torch.zeros(100, dtype=torch.float64, device="cuda")
    y = torch.zeros(100, dtype=torch.float64, device="cuda")
    x[37] = float("nan")
    p = NufftPlan(2, (16, 16), eps=1e-5)
    with pytest.raises(GbnError) as ei:
        p.set_points([x, y])
    assert ei.value.status == 1 and "non-finite" in str(ei.value)
    with pytest.raises(GbnError):
        p.type2(torch.zeros((1, 16, 16, 1), dtype=torch.complex64, device="cuda"))


def test_shape_and_dtype_errors():
    p = NufftPlan(2, (16, 16), n_coil=2, eps=1e-5)
    x = torch.zeros(10, dtype=torch.float64, device="cuda")
    p.set_points([x, x])
    with pytest.raises(ValueError):
        p.type2(torch.zeros((1, 16, 15, 2), dtype=torch.complex64, device="cuda"))
    with pytest.raises(TypeError):
        p.type2(torch.zeros((1, 16, 16, 2), dtype=torch.complex128, device="cuda"))
    with pytest.raises(ValueError):
        p.set_points([x, x], traj_offsets=[0, 5])


def test_empty_trajectory():
    p = NufftPlan(2, (16, 16), eps=1e-5)
    e = torch.zeros(0, dtype=torch.float64, device="cuda")
    p.set_points([e, e])
    out = p.type1(torch.zeros((0, 1), dtype=torch.complex64, device="cuda"))
    assert out.shape == (1, 16, 16, 1) and torch.count_nonzero(out) == 0
    k = p.type2(torch.ones((1, 16, 16, 1), dtype=torch.complex64, device="cuda"))
    assert k.shape == (0, 1)


def test_spread_kernel_count_reported():
    """plan.info()['spread_kernels'] counts the kernels the last spread launched: the 3-D
    compensated instance appears when dense tiles exist, the split-tile zeroing when the grid
    is not cleared by a memset."""
    rng = np.random.default_rng(26)
    xs = rng.uniform(-np.pi, np.pi, (3, 20000)) * 0.1          # everything in the centre
    p3 = NufftPlan(3, (16, 16, 16), n_coil=8, eps=1e-6, max_nspread=6, dense_tile_samples=64)
    p3.set_points([cuda(v) for v in xs])
    assert p3.info()["spread_kernels"] == 0
    p3.type1(cuda(cvec(rng, (20000, 8))))
    assert p3.info()["dense_subproblems"] > 0 and p3.info()["spread_kernels"] >= 2
    p3n = NufftPlan(3, (16, 16, 16), n_coil=8, eps=1e-6, max_nspread=6, dense_tile_samples=-1)
    p3n.set_points([cuda(v) for v in xs])
    p3n.type1(cuda(cvec(rng, (20000, 8))))
    assert p3n.info()["spread_kernels"] == p3.info()["spread_kernels"] - 1
