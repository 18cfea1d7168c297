"""GPU: ESPIRiT coil maps (mripy_gb300.espirit, the gbn_espirit_eigen kernel) against the
FP64 oracle restatement of espirit/espirit_func.py and against known synthetic maps."""
import numpy as np
import pytest
import torch

from mripy_gb300 import espirit as E
from mripy_gb300 import synth
from oracle import espirit_oracle as EO

pytestmark = pytest.mark.gpu


def _calib(shape, nc, calib, rng):
    S = synth.coil_maps(shape, nc, rng)
    x = synth.ellipse_phantom(shape[0], rng) if len(shape) == 2 else synth.ellipsoid_phantom(shape[0], rng)
    d = len(shape)
    ksp = EO.ft_forward(x[..., None] * S, tuple(range(d)))
    sl = tuple(slice(n // 2 - calib // 2, n // 2 - calib // 2 + calib) for n in shape)
    return ksp[sl], S, x


def _agreement(v, ref, keep):
    """per-pixel |<v, ref>| / (|v| |ref|) over the kept pixels"""
    num = np.abs(np.sum(v * np.conj(ref), axis=-1))
    den = np.linalg.norm(v, axis=-1) * np.linalg.norm(ref, axis=-1) + 1e-30
    return (num / den)[keep]


@pytest.mark.parametrize("nc,nsv", [(8, 40), (3, 7), (32, 5), (1, 4)])
def test_eigen_kernel_matches_eigh(nc, nsv):
    rng = np.random.default_rng(60)
    P = 3000
    # a dominant direction per pixel plus noise: a clear eigen gap
    u = rng.standard_normal((P, 1, nc)) + 1j * rng.standard_normal((P, 1, nc))
    coef = rng.standard_normal((P, nsv, 1)) + 1j * rng.standard_normal((P, nsv, 1))
    A = coef * u + 0.1 * (rng.standard_normal((P, nsv, nc)) + 1j * rng.standard_normal((P, nsv, nc)))
    A = A.astype(np.complex64)
    v, s = E.espirit_eigen(torch.from_numpy(A).cuda(), n_iter=64)
    v_ref, s_ref = EO.eigen_pixels(A.astype(np.complex128))
    assert np.allclose(s.cpu().numpy(), s_ref, rtol=1e-4)
    assert np.abs(v.cpu().numpy() - v_ref).max() < 1e-4          # same canonical phase
    assert np.allclose(np.linalg.norm(v.cpu().numpy(), axis=-1), 1.0, atol=1e-5)


def test_eigen_kernel_zero_pixels_and_errors():
    a = torch.zeros((5, 3, 4), dtype=torch.complex64, device="cuda")
    v, s = E.espirit_eigen(a)
    assert torch.count_nonzero(v) == 0 and torch.count_nonzero(s) == 0
    with pytest.raises(RuntimeError):
        E.espirit_eigen(torch.zeros((2, 3, 33), dtype=torch.complex64, device="cuda"))


@pytest.mark.parametrize("pad_before", [0, 1])
def test_espirit_2d_matches_oracle(pad_before):
    rng = np.random.default_rng(61)
    shape, nc = (64, 64), 6
    xcrop, S, x = _calib(shape, nc, 24, rng)
    vg, sg, info = E.espirit_nd(xcrop, shape + (nc,), hkwin_shape=(16, 16), pad_before_espirit=pad_before,
                                return_info=True)
    vr, sr, iref = EO.espirit(xcrop, shape + (nc,), hkwin_shape=(16, 16), pad_before_espirit=pad_before,
                              return_info=True)
    assert info["nsv"] == iref["nsv"]
    assert np.allclose(info["singular_values"], iref["singular_values"], rtol=1e-4,
                       atol=1e-5 * iref["singular_values"][0])
    keep = sr > 0.05
    assert np.linalg.norm(sg[keep] - sr[keep]) / np.linalg.norm(sr[keep]) < 1e-3
    assert np.quantile(_agreement(vg, vr, keep), 0.01) > 0.999
    # and the maps are the true ones up to a phase per pixel inside the object
    inside = np.abs(x) > 0.2 * np.abs(x).max()
    assert np.median(_agreement(vg, S, inside)) > 0.95


def test_espirit_2d_torch_in_torch_out():
    rng = np.random.default_rng(62)
    shape, nc = (32, 32), 4
    xcrop, S, x = _calib(shape, nc, 20, rng)
    vg, sg = E.espirit_2d(torch.from_numpy(xcrop.astype(np.complex64)).cuda(), shape + (nc,), hkwin_shape=(12, 12))
    assert vg.is_cuda and vg.shape == shape + (nc,) and sg.shape == shape
    vn, sn = E.espirit_2d(xcrop, shape + (nc,), hkwin_shape=(12, 12))
    assert isinstance(vn, np.ndarray) and vn.dtype == np.complex128
    assert np.abs(vg.cpu().numpy() - vn).max() < 1e-5


def test_espirit_3d_matches_oracle():
    rng = np.random.default_rng(63)
    shape, nc = (32, 32, 32), 4
    xcrop, S, x = _calib(shape, nc, 16, rng)
    vg, sg, info = E.espirit_nd(xcrop, shape + (nc,), hkwin_shape=(8, 8, 8), return_info=True)
    vr, sr, iref = EO.espirit(xcrop, shape + (nc,), hkwin_shape=(8, 8, 8), return_info=True)
    assert info["nsv"] == iref["nsv"]
    keep = sr > 0.05
    assert np.linalg.norm(sg[keep] - sr[keep]) / np.linalg.norm(sr[keep]) < 1e-3
    assert np.quantile(_agreement(vg, vr, keep), 0.01) > 0.999


def test_espirit_3d_wide_calibration_matches_oracle():
    """A 3-D calibration whose Hankel matrix (512 x 8788) takes the FP32 Gram product."""
    rng = np.random.default_rng(64)
    shape, nc = (32, 32, 32), 4
    xcrop, S, x = _calib(shape, nc, 20, rng)
    vg, sg, info = E.espirit_nd(xcrop, shape + (nc,), hkwin_shape=(8, 8, 8), return_info=True)
    vr, sr, iref = EO.espirit(xcrop, shape + (nc,), hkwin_shape=(8, 8, 8), return_info=True)
    assert info["nsv"] == iref["nsv"]
    s0 = iref["singular_values"][0]
    kept = iref["singular_values"] > 0.2 * s0
    assert np.allclose(info["singular_values"][kept], iref["singular_values"][kept], rtol=1e-4)
    keep = sr > 0.05
    assert np.linalg.norm(sg[keep] - sr[keep]) / np.linalg.norm(sr[keep]) < 1e-3
    assert np.quantile(_agreement(vg, vr, keep), 0.01) > 0.999
