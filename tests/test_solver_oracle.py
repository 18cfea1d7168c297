"""The solver oracle (FP64 numpy restatement of DWTnd('haar'), the soft threshold, IST_32,
FIST_32 and linear CG) pinned by known answers of the published Haar transform.  CPU only."""
import numpy as np
import pytest

from oracle import solver_oracle as SO

R2 = 1.0 / np.sqrt(2.0)


def test_haar_1d_level2_known_answer():
    # pywt.wavedec([1..8], 'haar', level=2) = [cA2, cD2, cD1] = [5, 13], [-2, -2], [-1/sqrt2] * 4
    c = SO.haar_dwt(np.arange(1.0, 9.0), 2, (0,))
    assert np.allclose(c, [5, 13, -2, -2, -R2, -R2, -R2, -R2], atol=1e-14)
    assert np.allclose(SO.haar_idwt(c, 2, (0,)), np.arange(1.0, 9.0), atol=1e-13)


def test_haar_2d_level1_block_layout():
    # one 2x2 block: aa = sum/2 at [0, 0]; 'ad' (detail along axis 1) at [0, 1]; 'da' at
    # [1, 0]; 'dd' at [1, 1] -- coeffs_to_array's placement of the level-1 details
    x = np.array([[1.0, 3.0], [5.0, 7.0]])
    c = SO.haar_dwt(x, 1, (0, 1))
    assert np.allclose(c, [[8.0, -2.0], [-4.0, 0.0]], atol=1e-14)


def test_haar_2d_level2_places_each_level():
    # a 4x4 image constant on 2x2 blocks has no level-1 details; level 2 acts on the
    # approximation block [0:2, 0:2] only
    blocks = np.array([[1.0, 2.0], [3.0, 4.0]])
    x = np.kron(blocks, np.ones((2, 2)))
    c = SO.haar_dwt(x, 2, (0, 1))
    assert np.allclose(c[2:, :], 0) and np.allclose(c[:, 2:], 0)
    # level-1 approximation = 2 * blocks; level 2 of that is blocks' 2-D Haar times 2
    assert np.allclose(c[:2, :2], 2 * SO.haar_dwt(blocks, 1, (0, 1)), atol=1e-13)
    assert np.isclose(c[0, 0], x.sum() / 4)


def test_haar_3d_orthonormal_and_invertible_over_leading_axes():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((8, 16, 4, 3)) + 1j * rng.standard_normal((8, 16, 4, 3))
    c = SO.haar_dwt(x, 2, (0, 1, 2))
    assert np.isclose(np.linalg.norm(c), np.linalg.norm(x), rtol=1e-13)
    assert np.allclose(SO.haar_idwt(c, 2, (0, 1, 2)), x, atol=1e-12)
    # the trailing axis is independent
    c0 = SO.haar_dwt(x[..., 1], 2, (0, 1, 2))
    assert np.allclose(c[..., 1], c0, atol=1e-13)


def test_haar_rejects_sizes_not_divisible():
    with pytest.raises(ValueError):
        SO.haar_dwt(np.zeros(6), 2, (0,))


def test_soft_threshold_reference_formula():
    rng = np.random.default_rng(1)
    x0 = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    a = np.abs(x0) - 0.5
    a[a < 0] = 0
    assert np.allclose(SO.soft_thresh(x0, 0.5), x0 / (np.abs(x0) + 1e-6) * a, atol=1e-15)


def test_cg_solves_spd_system():
    rng = np.random.default_rng(2)
    B = rng.standard_normal((20, 12)) + 1j * rng.standard_normal((20, 12))
    H = B.conj().T @ B
    xt = rng.standard_normal(12) + 1j * rng.standard_normal(12)
    x, norms = SO.cg(lambda v: H @ v, H @ xt, 12)
    assert np.allclose(x, xt, atol=1e-8)
    assert norms[-1] < 1e-6 * norms[0]


def test_ist_fista_first_iterate_is_the_prox_of_the_gradient_step():
    # with N = 0 and step 1 the first IST and FISTA iterates are prox(rhs)
    rng = np.random.default_rng(3)
    rhs = rng.standard_normal((8, 8)) + 1j * rng.standard_normal((8, 8))
    ref = SO.prox_haar(rhs, 0.3, 2, (0, 1))
    assert np.allclose(SO.ist(lambda v: 0 * v, rhs, 1, 1.0, 0.3, 2, (0, 1)), ref, atol=1e-13)
    assert np.allclose(SO.fista(lambda v: 0 * v, rhs, 1, 1.0, 0.3, 2, (0, 1)), ref, atol=1e-13)


def test_pipe_menon_fixed_point_and_radial_density():
    from mripy_gb300 import synth
    import oracle as O
    kx, ky = synth.radial_2d(32, 64)
    coords = (2 * np.pi * kx, 2 * np.pi * ky)
    shape = (32, 32)
    w = SO.pipe_menon_dcf(coords, shape, 30)
    assert np.isclose(w.mean(), 1.0)
    # fixed point: interp(spread(w)) is the same at every sample
    ns, nf, tau = O.grid_params(2, 32, 32, eps=1e-5)
    cw = np.abs(O.interp(coords, O.spread(coords, w[None].astype(np.complex128), tau, ns, nf), tau, ns)[0])
    assert np.std(cw) / np.mean(cw) < 0.05
    # radial sampling density falls as 1/|k|: away from the centre the weights grow with |k|
    r = np.hypot(kx, ky)
    mid = (r > 0.1) & (r < 0.4)
    assert np.corrcoef(r[mid], w[mid])[0, 1] > 0.95
