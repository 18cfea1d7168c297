"""The pruned FFT of the composite calls (fft_variant 2, gbn_fft_band): the trailing axes are
transformed only on the grid planes inside the image band along x, the x pass on every plane.

Covered: the band transform after the pad (GBN_BAND_INPUT) against the full transform on the
whole grid; before the crop (GBN_BAND_OUTPUT) against the full transform on the band the crop
reads; even and odd image sizes (two or three band-run lengths), one instance and several
trajectory groups x coils, 2-D and 3-D; type 1, type 2 and type 21 with the pruned transform
against the same plan with the full one, and against the FP64 oracle; the library's choice by
grid size; argument errors.

Tolerance: 2e-6 relative L2 between the pruned and the full transform (the same cuFFT sums in
another order), TOL_REF = 2e-5 against the FP64 oracle.
"""
import numpy as np
import pytest
import torch

import oracle as O
from mripy_gb300 import _native as N
from mripy_gb300.plan import NufftPlan, Tuning

pytestmark = pytest.mark.gpu

TOL_FFT = 2e-6
TOL_REF = 2e-5


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def cvec(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


def rel(a, b):
    return float((a - b).norm() / b.norm())


def _plans(dim, shape, nc, n_traj, xs, offsets=None, eps=5e-6):
    out = []
    for fv in (2, 1):
        p = NufftPlan(dim, shape, n_coil=nc, n_traj=n_traj, eps=eps, max_nspread=6 if dim == 3 else None,
                      tuning=Tuning(fft_variant=fv))
        p.set_points([cuda(v) for v in xs], traj_offsets=offsets)
        assert p.info()["fft_variant"] == fv
        out.append(p)
    return out


def _band_mask(p):
    """Boolean mask of the grid cells inside the image band along every axis."""
    nf, m = p.info()["nf"], p.shape
    axes = []
    for n, mm in zip(nf, m):
        a = np.zeros(n, bool)
        a[:mm - mm // 2] = True
        a[n - mm // 2:] = True
        axes.append(a)
    mask = axes[0]
    for a in axes[1:]:
        mask = np.logical_and.outer(mask, a)
    return torch.from_numpy(mask).cuda()


@pytest.mark.parametrize("dim,shape,nc,n_traj", [(3, (20, 18, 22), 3, 2), (3, (21, 17, 19), 2, 1),
                                                 (3, (21, 16, 16), 1, 3), (2, (40, 36), 4, 2),
                                                 (2, (33, 29), 1, 1)])
def test_band_transform_against_full(dim, shape, nc, n_traj):
    rng = np.random.default_rng(60 + dim + nc)
    M = 500
    xs = rng.uniform(-np.pi, np.pi, (dim, M * n_traj))
    off = [M * k for k in range(n_traj + 1)]
    pb, pf = _plans(dim, shape, nc, n_traj, xs, off)
    img = cuda(cvec(rng, (n_traj,) + shape + (nc,)))
    for direction in (N.GBN_FFT_FORWARD, N.GBN_FFT_INVERSE):
        # after the pad: the band transform is the full transform on the whole grid
        g1 = pb.pad_deapod(img, pb.grid()).clone()
        g2 = g1.clone()
        pb.fft_band(g1, direction, N.GBN_BAND_INPUT)
        pf.fft(g2, direction)
        assert rel(g1, g2) < TOL_FFT
        # before the crop: equal on the band cells the crop reads
        g = cuda(cvec(rng, tuple(g1.shape)))
        h1, h2 = g.clone(), g.clone()
        pb.fft_band(h1, direction, N.GBN_BAND_OUTPUT)
        pf.fft(h2, direction)
        mask = _band_mask(pb)
        assert rel(h1[:, mask], h2[:, mask]) < TOL_FFT
        i1 = pb.crop_deapod(h1)
        i2 = pf.crop_deapod(h2)
        assert rel(i1, i2) < TOL_FFT
    pb.status()
    pb.close()
    pf.close()


@pytest.mark.parametrize("dim,shape,nc", [(3, (24, 20, 22), 4), (3, (19, 21, 17), 8), (2, (48, 44), 8)])
def test_composite_calls_pruned_against_full_and_oracle(dim, shape, nc):
    rng = np.random.default_rng(70 + nc)
    M, n_traj = 4000, 2
    xs = rng.uniform(-np.pi, np.pi, (dim, M))
    xs[:, :M // 3] *= 0.1
    off = [0, 1700, M]
    pb, pf = _plans(dim, shape, nc, n_traj, xs, off)
    img = cvec(rng, (n_traj,) + shape + (nc,))
    c = cvec(rng, (M, nc))
    dcf = cuda(rng.uniform(0.5, 1.5, M).astype(np.float32))
    k2b, k2f = pb.type2(cuda(img)), pf.type2(cuda(img))
    assert rel(k2b, k2f) < TOL_FFT * 5
    k1b, k1f = pb.type1(cuda(c)), pf.type1(cuda(c))
    assert rel(k1b, k1f) < TOL_FFT * 5
    k21b, k21f = pb.type21(cuda(img), dcf=dcf), pf.type21(cuda(img), dcf=dcf)
    assert rel(k21b, k21f) < TOL_FFT * 5
    pb.status()
    for g in range(n_traj):
        a, b = off[g], off[g + 1]
        ref2 = O.nufft_type2(tuple(x[a:b] for x in xs), img[g].astype(np.complex128), shape, eps=5e-6)
        assert float(np.linalg.norm(k2b[a:b].cpu().numpy() - ref2) / np.linalg.norm(ref2)) < TOL_REF
        ref1 = O.nufft_type1(tuple(x[a:b] for x in xs), c[a:b].astype(np.complex128), shape, eps=5e-6)
        assert float(np.linalg.norm(k1b[g].cpu().numpy() - ref1) / np.linalg.norm(ref1)) < TOL_REF
    pb.close()
    pf.close()


def test_library_choice_and_arguments():
    """Pruned by default on 3-D grids of >= 2^21 cells per instance; full on smaller ones and in 2-D."""
    rng = np.random.default_rng(75)
    xs3 = rng.uniform(-np.pi, np.pi, (3, 100))
    big = NufftPlan(3, (64, 64, 64), n_coil=2, eps=5e-6, max_nspread=6)
    assert big.info()["nf"] == (128, 128, 128) and big.info()["fft_variant"] == 2
    small = NufftPlan(3, (32, 32, 32), n_coil=2, eps=5e-6, max_nspread=6)
    assert small.info()["fft_variant"] == 1
    flat = NufftPlan(2, (512, 512), n_coil=8, eps=5e-6)
    assert flat.info()["fft_variant"] == 1
    off = NufftPlan(3, (64, 64, 64), n_coil=2, eps=5e-6, max_nspread=6, tuning=Tuning(fft_variant=1))
    assert off.info()["fft_variant"] == 1
    big.set_points([cuda(v) for v in xs3])
    with pytest.raises(N.GbnError):
        big.fft_band(big.grid(), N.GBN_FFT_FORWARD, 3)
    with pytest.raises(N.GbnError):
        NufftPlan(3, (16, 16, 16), n_coil=1, eps=5e-6, max_nspread=6, tuning=Tuning(fft_variant=3))
    for p in (big, small, flat, off):
        p.close()
