"""GPU: the solver kernels through the C ABI against the FP64 solver oracle -- the Haar
transform and its prox (tile kernels), CG (gbn_cg_sense) and IST/FISTA (gbn_ista_haar)
with the normal operators of NUFFT2d / joint2operators(espirit, NUFFT)."""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import solver_oracle as SO
from mripy_gb300 import operators as ops
from mripy_gb300 import plan as P
from mripy_gb300 import solvers, synth

pytestmark = pytest.mark.gpu

EPS_OP = 1e-5   # the operator classes' eps


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _crand(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


HAAR_CASES = [
    ((64,), (0,), 3),
    ((64,), (0,), 0),
    ((32, 48, 3), (0, 1), 4),
    ((2, 64, 64), (1, 2), 6),
    ((16, 16, 32, 2), (0, 1, 2), 4),
    ((3, 8, 8, 8), (1, 2, 3), 1),
    ((24, 40), (0, 1), 3),
]


@pytest.mark.parametrize("shape,axes,level", HAAR_CASES)
def test_haar_dwt_matches_oracle_layout_and_inverts(shape, axes, level):
    rng = np.random.default_rng(40)
    x = _crand(rng, shape)
    xt = torch.from_numpy(x).cuda()
    c = P.haar_dwt(xt, level, axes)
    ref = SO.haar_dwt(x.astype(np.complex128), level, axes)
    assert rel(c, ref) < 1e-6
    back = P.haar_dwt(c, level, axes, inverse=True)
    assert rel(back, x) < 1e-6


@pytest.mark.parametrize("shape,axes,level", HAAR_CASES)
def test_prox_haar_matches_oracle(shape, axes, level):
    rng = np.random.default_rng(41)
    x = _crand(rng, shape)
    th = float(np.median(np.abs(x)))
    out = P.prox_haar(torch.from_numpy(x).cuda(), th, level, axes)
    ref = SO.prox_haar(x.astype(np.complex128), th, level, axes)
    assert rel(out, ref) < 1e-5
    # in place gives the same
    xt = torch.from_numpy(x).cuda()
    P.prox_haar(xt, th, level, axes, out=xt)
    assert torch.equal(xt, out)


def test_haar_rejects_bad_shapes():
    x = torch.zeros(24, 40, dtype=torch.complex64, device="cuda")
    with pytest.raises(RuntimeError):
        P.haar_dwt(x, 4, (0, 1))          # 24 is not a multiple of 16
    with pytest.raises(RuntimeError):
        P.haar_dwt(torch.zeros(128, 128, 128, dtype=torch.complex64, device="cuda"), 5, (0, 1, 2))  # 32^3 tiles
    with pytest.raises(NotImplementedError):
        P.haar_dwt(x, 1, (0, 2))


def test_dwtnd_class_numpy_and_cuda():
    rng = np.random.default_rng(42)
    x = rng.standard_normal((16, 16, 16, 1)) + 1j * rng.standard_normal((16, 16, 16, 1))
    w = solvers.DWTnd("haar", level=3, axes=(0, 1, 2))
    c = w.backward(x)
    assert isinstance(c, np.ndarray) and c.dtype == np.complex128
    assert rel(c, SO.haar_dwt(x, 3, (0, 1, 2))) < 1e-6
    assert rel(w.forward(c), x) < 1e-6
    ct = w.backward(torch.from_numpy(x.astype(np.complex64)).cuda())
    assert ct.is_cuda and rel(ct, c) < 1e-6


def test_soft_threshold_kernel_matches_formula():
    rng = np.random.default_rng(43)
    x = _crand(rng, (1000,))
    out = solvers.prox_l1_soft_thresh2(torch.from_numpy(x).cuda(), 0.8)
    assert rel(out, SO.soft_thresh(x.astype(np.complex128), 0.8)) < 1e-6


# ---------------------------------------------------------------- CG
# Samples uniform over the whole k-space square: the normal operator is well conditioned,
# so FP32 and FP64 iterations agree to ~1e-7 (an FP32 restatement of the loop was checked on
# the CPU).  A radial trajectory leaves the square's corners unsampled; the near-null space
# that leaves is filled by rounding, and FP32 and FP64 CG iterates then differ by ~2e-2 for
# any FP32 implementation (the same CPU restatement shows it), which says nothing about the
# kernels.
def _uniform_coords(rng, M=3072):
    return tuple(rng.uniform(-np.pi, np.pi, M) for _ in range(2))


def _nufft2d_problem(rng, shape=(32, 32), nc=2):
    coords = _uniform_coords(rng)
    x = synth.ellipse_phantom(shape[0], rng)[..., None] * np.ones(nc)
    y = O.nufft_type2(coords, x.astype(np.complex128), shape, eps=EPS_OP)
    nft = ops.NUFFT2d(shape)
    nft.set_ktraj(*coords)
    return nft, coords, y


def _normal64(coords, shape):
    return lambda v: O.nufft_type21(coords, v, shape, eps=EPS_OP)


@pytest.mark.parametrize("use_graph", [True, False])
def test_cg_nufft2d_matches_fp64_cg(use_graph):
    rng = np.random.default_rng(44)
    shape = (32, 32)
    nft, coords, y = _nufft2d_problem(rng, shape)
    x, norms = solvers.cg_sense(nft, torch.tensor(y.astype(np.complex64), device="cuda"), n_iter=10,
                                use_graph=use_graph)
    b = O.nufft_type1(coords, y, shape, eps=EPS_OP)
    x64, n64 = SO.cg(_normal64(coords, shape), b, 10)
    assert rel(x, x64) < 1e-4
    assert np.allclose(norms.cpu().numpy(), n64, rtol=1e-3)


def test_cg_graph_and_direct_launches_agree():
    # the solver's own reductions are in a fixed order; the spread's split tiles (several
    # work items per dense tile) merge with float atomics, so runs agree to rounding only
    rng = np.random.default_rng(45)
    shape = (32, 32)
    nft, coords, y = _nufft2d_problem(rng, shape)
    yt = torch.tensor(y.astype(np.complex64), device="cuda")
    xa, na = solvers.cg_sense(nft, yt, n_iter=6, use_graph=True)
    xb, nb = solvers.cg_sense(nft, yt, n_iter=6, use_graph=False)
    xc, nc_ = solvers.cg_sense(nft, yt, n_iter=6, use_graph=True)     # replays the cached graph
    assert rel(xa, xb) < 1e-4 and rel(xc, xa) < 1e-4
    assert np.allclose(na.cpu().numpy(), nb.cpu().numpy(), rtol=1e-4)
    assert np.allclose(nc_.cpu().numpy(), na.cpu().numpy(), rtol=1e-4)


def test_cg_warm_start_continues_the_iteration():
    rng = np.random.default_rng(46)
    shape = (32, 32)
    nft, coords, y = _nufft2d_problem(rng, shape)
    p = nft.plan(2)
    b = nft.backward(torch.tensor(y.astype(np.complex64), device="cuda")).reshape((1,) + shape + (2,)).contiguous()
    x4, _ = p.cg(b, 4)
    x8, _ = p.cg(b, 4, x0=x4)
    b64 = O.nufft_type1(coords, y, shape, eps=EPS_OP)
    ref, _ = SO.cg(_normal64(coords, shape), b64, 4, x0=x4[0].cpu().numpy().astype(np.complex128))
    assert rel(x8[0], ref) < 1e-4


def test_cg_sense_native_matches_fp64_cg_with_operator_eps():
    rng = np.random.default_rng(47)
    shape, nc = (32, 32), 4
    coords = _uniform_coords(rng)
    S = synth.coil_maps(shape, nc, rng)
    x = synth.ellipse_phantom(shape[0], rng)
    y = O.nufft_type2(coords, (x[..., None] * S).astype(np.complex128), shape, eps=EPS_OP)
    nft = ops.NUFFT2d(shape)
    nft.set_ktraj(*coords)
    A = ops.joint2operators(ops.espirit(S), nft)
    xg, norms = solvers.cg_sense(A, torch.tensor(y.astype(np.complex64), device="cuda"), n_iter=8)

    def normal(v):
        return np.sum(np.conj(S) * O.nufft_type21(coords, v[..., None] * S, shape, eps=EPS_OP), axis=-1)
    b = np.sum(np.conj(S) * O.nufft_type1(coords, y, shape, eps=EPS_OP), axis=-1)
    x64, n64 = SO.cg(normal, b, 8)
    assert rel(xg.reshape(shape), x64) < 1e-4
    assert np.allclose(norms.cpu().numpy(), n64, rtol=1e-3)


def test_solver_graph_follows_new_points():
    rng = np.random.default_rng(48)
    shape = (32, 32)
    nft, coords, y = _nufft2d_problem(rng, shape)
    p = nft.plan(2)
    b = torch.tensor(_crand(rng, (1,) + shape + (2,)), device="cuda")
    p.cg(b, 3)                                           # captures the iteration graph
    c2 = _uniform_coords(rng, 2500)
    p.set_points([torch.tensor(c, device="cuda") for c in c2])
    x, _ = p.cg(b, 3)
    ref, _ = SO.cg(_normal64(c2, shape), b[0].cpu().numpy().astype(np.complex128), 3)
    assert rel(x[0], ref) < 1e-4


# ---------------------------------------------------------------- IST / FISTA
@pytest.mark.parametrize("fista", [False, True])
@pytest.mark.parametrize("level", [0, 2])
def test_ist_fista_nufft2d_match_fp64(fista, level):
    rng = np.random.default_rng(49)
    shape = (32, 32)
    nft, coords, y = _nufft2d_problem(rng, shape)
    yt = torch.tensor(y.astype(np.complex64), device="cuda")
    T = solvers.DWTnd("haar", level=level, axes=(0, 1)) if level else None
    wrap = solvers.FIST_wrap if fista else solvers.IST_wrap
    x = wrap(nft, T, yt, 6, 0.5, 1e-3)
    b = O.nufft_type1(coords, y, shape, eps=EPS_OP)
    solve = SO.fista if fista else SO.ist
    ref = solve(_normal64(coords, shape), b, 6, 0.5, 1e-3, level, (0, 1))
    assert x.shape == (32, 32, 2)
    assert rel(x, ref) < 1e-4


def test_fista_sense_numpy_in_numpy_out():
    rng = np.random.default_rng(50)
    shape, nc = (32, 32), 3
    coords = _uniform_coords(rng)
    S = synth.coil_maps(shape, nc, rng)
    x = synth.ellipse_phantom(shape[0], rng)
    y = O.nufft_type2(coords, (x[..., None] * S).astype(np.complex128), shape, eps=EPS_OP)
    nft = ops.NUFFT2d(shape)
    nft.set_ktraj(*coords)
    A = ops.joint2operators(ops.espirit(S), nft)
    xr = solvers.FIST_wrap(A, solvers.DWTnd("haar", level=3, axes=(0, 1)), y, 5, 0.5, 2e-4)
    assert isinstance(xr, np.ndarray) and xr.shape == shape + (1,)

    def normal(v):
        return np.sum(np.conj(S) * O.nufft_type21(coords, v * S, shape, eps=EPS_OP), axis=-1, keepdims=True)
    b = np.sum(np.conj(S) * O.nufft_type1(coords, y, shape, eps=EPS_OP), axis=-1, keepdims=True)
    ref = SO.fista(normal, b, 5, 0.5, 2e-4, 3, (0, 1))
    assert rel(xr, ref) < 1e-4


# ---------------------------------------------------------------- density compensation
def test_pipe_menon_dcf_2d_ragged_groups_match_oracle():
    kx, ky = synth.golden_radial_2d(60, 64)
    coords = (2 * np.pi * kx, 2 * np.pi * ky)
    offsets = [0, 40 * 64, 40 * 64, 60 * 64]         # three frames: 40, 0 and 20 spokes
    plan = P.NufftPlan(2, (32, 32), n_coil=1, n_traj=3, eps=EPS_OP)
    plan.set_points([torch.tensor(c, device="cuda") for c in coords], traj_offsets=offsets)
    w = plan.pipe_menon_dcf(12)
    ref = SO.pipe_menon_dcf(coords, (32, 32), 12, eps=EPS_OP, offsets=offsets)
    assert rel(w, ref) < 1e-4
    wn = w.cpu().numpy()
    assert np.isclose(wn[:offsets[1]].mean(), 1.0, rtol=1e-5) and np.isclose(wn[offsets[2]:].mean(), 1.0, rtol=1e-5)


def test_pipe_menon_dcf_3d_operator():
    kk = synth.centre_out_radial_3d(300, 16)
    nft = ops.NUFFT3d((16, 16, 16))
    nft.normalize_set_ktraj(np.stack(kk))
    coords = tuple(np.asarray(k.cpu() if isinstance(k, torch.Tensor) else k, dtype=np.float64)
                   for k in nft._k[:3])
    w = nft.pipe_menon_dcf(10)
    ref = SO.pipe_menon_dcf(coords, (16, 16, 16), 10, eps=EPS_OP)
    assert rel(w, ref) < 1e-4
    assert nft.dcf is w


def test_pipe_menon_dcf_needs_one_coil():
    plan = P.NufftPlan(2, (16, 16), n_coil=2, eps=EPS_OP)
    plan.set_points([torch.zeros(10, dtype=torch.float64, device="cuda")] * 2)
    with pytest.raises(RuntimeError):
        plan.pipe_menon_dcf(3)


def test_fista_ragged_frames_match_per_frame_oracle():
    """gbn_ista_haar over two trajectory groups of different sizes: the normal operator is
    block-diagonal over frames and the Haar tiles never cross an image, so each frame's
    iterate equals a separate FP64 FISTA on that frame."""
    rng = np.random.default_rng(51)
    shape, nc = (32, 32), 2
    counts = [3000, 1700]
    off = [0, counts[0], counts[0] + counts[1]]
    xs = rng.uniform(-np.pi, np.pi, (2, off[-1]))
    p = P.NufftPlan(2, shape, n_coil=nc, n_traj=2, eps=EPS_OP)
    p.set_points([torch.tensor(v, device="cuda") for v in xs], traj_offsets=off)
    rhs = _crand(rng, (2,) + shape + (nc,))
    x = p.ista(torch.from_numpy(rhs).cuda(), 5, 0.5, 1e-2, 2, fista=True)
    for g in range(2):
        a, b = off[g], off[g + 1]
        ref = SO.fista(_normal64((xs[0][a:b], xs[1][a:b]), shape), rhs[g].astype(np.complex128), 5, 0.5, 1e-2,
                       2, (0, 1))
        assert rel(x[g], ref) < 1e-4


# ---------------------------------------------------------------- ADMM (pics/CS_MRI_solvers_func.py:321-333)
def test_admm_sense_cuda_matches_fp64_admm_on_oracle_operators():
    from mripy_gb300 import admm
    rng = np.random.default_rng(60)
    shape, nc = (32, 32), 3
    coords = _uniform_coords(rng)
    S = synth.coil_maps(shape, nc, rng)
    x = synth.ellipse_phantom(shape[0], rng)
    y = O.nufft_type2(coords, (x[..., None] * S).astype(np.complex128), shape, eps=EPS_OP)
    nft = ops.NUFFT2d(shape)
    nft.set_ktraj(*coords)
    A = ops.joint2operators(ops.espirit(S), nft)
    yt = torch.from_numpy(y.astype(np.complex64)).cuda()
    xr = admm.ADMM_l2Afxnb_l1x(A.forward, A.backward, yt, 4, 0.5, 0.01, 1.0)
    assert isinstance(xr, torch.Tensor) and xr.is_cuda and xr.shape == shape + (1,)

    def Af(v):
        return O.nufft_type2(coords, v * S, shape, eps=EPS_OP)

    def AHf(k):
        return np.sum(np.conj(S) * O.nufft_type1(coords, k, shape, eps=EPS_OP), axis=-1, keepdims=True)
    ref = admm.ADMM_l2Afxnb_l1x(Af, AHf, y, 4, 0.5, 0.01, 1.0)
    assert rel(xr, ref) < 1e-3
