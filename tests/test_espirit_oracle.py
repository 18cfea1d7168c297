"""The ESPIRiT oracle (FP64 numpy restatement of espirit/espirit_func.py) pinned by known
answers of its pieces and by recovering known coil maps from synthetic Cartesian data.  CPU."""
import numpy as np

from mripy_gb300 import synth
from oracle import espirit_oracle as EO


def cartesian_calibration(shape, nc, calib, rng, seed_img=None):
    """Multi-coil k-space of an ellipse phantom times smooth maps (the reference's FFT
    convention) and its centred calibration block."""
    S = synth.coil_maps(shape, nc, rng)
    if len(shape) == 2:
        x = synth.ellipse_phantom(shape[0], rng)
    else:
        x = synth.ellipsoid_phantom(shape[0], rng)
    d = len(shape)
    ksp = EO.ft_forward(x[..., None] * S, tuple(range(d)))
    sl = tuple(slice(n // 2 - calib // 2, n // 2 - calib // 2 + calib) for n in shape)
    return ksp[sl], S, x


def test_hankel_matrix_entries():
    rng = np.random.default_rng(0)
    a = rng.standard_normal((6, 7, 2)) + 1j * rng.standard_normal((6, 7, 2))
    H, moves = EO.hankel_matrix(a, (3, 4))
    assert moves == (4, 4) and H.shape == (12, 32)
    # row = window position (i0, i1), column = (m0, m1, coil): a[i0 + m0, i1 + m1, coil]
    for i0 in range(3):
        for i1 in range(4):
            for m0 in range(4):
                for m1 in range(4):
                    for c in range(2):
                        assert H[i0 * 4 + i1, (m0 * 4 + m1) * 2 + c] == a[i0 + m0, i1 + m1, c]


def test_hamming_and_pad_known_values():
    assert np.allclose(EO._hamming(5), [0.08, 0.54, 1.0, 0.54, 0.08])
    w = EO.hamming_nd((5, 3))
    assert np.allclose(w, np.sqrt(np.outer(EO._hamming(5), EO._hamming(3))))
    p = EO.pad_center(np.ones((3, 2)), (8, 5))
    # rows 8//2 - 3//2 = 3 .. 5, columns 5//2 - 2//2 = 1 .. 2
    assert p.sum() == 6 and p[3:6, 1:3].all()


def test_kept_count_is_the_last_index_above_threshold():
    s = np.array([10.0, 5.0, 2.5, 1.9, 0.1])
    assert EO.kept_count(s, 0.2) == 2


def test_espirit_2d_recovers_coil_maps():
    rng = np.random.default_rng(3)
    shape, nc = (64, 64), 4
    xcrop, S, x = cartesian_calibration(shape, nc, 24, rng)
    Vim, sim = EO.espirit(xcrop, shape + (nc,), hkwin_shape=(16, 16))
    inside = np.abs(x) > 0.2 * np.abs(x).max()
    corr = np.abs(np.sum(Vim * np.conj(S), axis=-1)) / np.linalg.norm(S, axis=-1)
    assert np.median(corr[inside]) > 0.95
    assert sim.max() == 1.0
