"""GPU: autograd gradients (image and trajectory) against FP64 NUDFT gradients and FP64
central finite differences; CG-SENSE and FISTA iterates against FP64 oracle operators."""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import solver_oracle as SO
from mripy_gb300 import autograd as AG
from mripy_gb300 import operators as ops
from mripy_gb300 import solvers, synth
from mripy_gb300.plan import NufftPlan

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_autograd_gradients_match_fp64_references():
    rng = np.random.default_rng(30)
    shape, nc = (32, 32), 3
    kx, ky = synth.vd_spiral_2d(4, 256)
    k0 = np.stack([kx, ky])                                   # cycles
    kp = k0 + rng.normal(0, 1e-3, k0.shape)
    M = k0.shape[1]
    x_true = (rng.standard_normal(shape + (nc,)) + 1j * rng.standard_normal(shape + (nc,)))
    y = O.nudft_type2((2 * np.pi * k0[0], 2 * np.pi * k0[1]), x_true, shape)           # (M, nc)
    x0 = x_true + 0.1 * (rng.standard_normal(x_true.shape) + 1j * rng.standard_normal(x_true.shape))

    plan = NufftPlan(2, shape, n_coil=nc, eps=5e-6)
    img = torch.tensor(x0.astype(np.complex64), device="cuda")[None].requires_grad_(True)
    k = torch.tensor(kp.astype(np.float32), device="cuda").requires_grad_(True)
    yt = torch.tensor(y.astype(np.complex64), device="cuda")
    c = AG.nufft_forward(img, 2 * np.pi * k, plan)
    loss = (c - yt).abs().pow(2).sum()
    loss.backward()

    xr = (2 * np.pi * kp[0], 2 * np.pi * kp[1])
    r = O.nudft_type2(xr, x0, shape) - y                       # exact residual
    # image gradient: 2 A^H r (exact adjoint sum)
    g_img = 2 * len(kp[0]) * O.nudft_type1(xr, r, shape)
    assert rel(img.grad[0], g_img) < 1e-3
    # trajectory gradient: d/dk = 2 pi * d/dx of sum |A(x)F - y|^2 = 2 pi * Re(conj(2r) dc/dx)
    g_x = O.nudft_type2_coord_grad(xr, x0, shape, 2 * r)
    g_k = 2 * np.pi * g_x.T
    assert rel(k.grad, g_k) < 1e-3
    # FP64 central finite differences (step 1e-6 in k) of the exact loss at a few samples
    def loss64(kk):
        cc = O.nudft_type2((2 * np.pi * kk[0], 2 * np.pi * kk[1]), x0, shape)
        return np.sum(np.abs(cc - y) ** 2)
    h = 1e-6
    scale = np.abs(g_k).max()
    for j in (0, 101, M - 1):
        for d in range(2):
            kpl, kmi = kp.copy(), kp.copy()
            kpl[d, j] += h
            kmi[d, j] -= h
            fd = (loss64(kpl) - loss64(kmi)) / (2 * h)
            assert abs(k.grad[d, j].item() - fd) <= 1e-3 * scale


def test_adjoint_function_backward():
    rng = np.random.default_rng(31)
    shape, M = (24, 24), 2000
    xs = torch.tensor(rng.uniform(-np.pi, np.pi, (2, M)), device="cuda")
    plan = NufftPlan(2, shape, eps=5e-6)
    c = torch.tensor((rng.standard_normal((M, 1)) + 1j * rng.standard_normal((M, 1))).astype(np.complex64),
                     device="cuda").requires_grad_(True)
    F = AG.nufft_adjoint(c, xs, plan)
    w = torch.tensor((rng.standard_normal(F.shape) + 1j * rng.standard_normal(F.shape)).astype(np.complex64),
                     device="cuda")
    loss = torch.real(torch.vdot(w.reshape(-1), F.reshape(-1)))
    loss.backward()
    # F = (1/M) A^H c, so d/dc Re<w, F> = (1/M) A w
    expect = plan.set_points([xs[0], xs[1]]).type2(w) / M
    assert rel(c.grad, expect) < 1e-5


def _small_sense_problem(rng, shape=(32, 32), nc=4, spokes=40, nread=64):
    kx, ky = synth.golden_radial_2d(spokes, nread)
    S = synth.coil_maps(shape, nc, rng)
    x = synth.ellipse_phantom(shape[0], rng)
    coords = (2 * np.pi * kx, 2 * np.pi * ky)
    y = O.nufft_type2(coords, (x[..., None] * S).astype(np.complex128), shape, eps=5e-6)
    return coords, S, x, y


def _cg_fp64(coords, S, y, shape, n_iter):
    def normal(v):
        return np.sum(np.conj(S) * O.nufft_type21(coords, v[..., None] * S, shape, eps=5e-6), axis=-1)
    b = np.sum(np.conj(S) * O.nufft_type1(coords, y, shape, eps=5e-6), axis=-1)
    x = np.zeros_like(b)
    r = b.copy()
    p = r.copy()
    rs = np.vdot(r, r).real
    for _ in range(n_iter):
        q = normal(p)
        a = rs / np.vdot(p, q).real
        x += a * p
        r -= a * q
        rn = np.vdot(r, r).real
        p = r + (rn / rs) * p
        rs = rn
    return x


@pytest.mark.parametrize("use_graph", [True, False])
def test_cg_sense_matches_fp64_cg(use_graph):
    rng = np.random.default_rng(32)
    shape = (32, 32)
    coords, S, x, y = _small_sense_problem(rng, shape)
    nft = ops.NUFFT2d(shape)
    nft.set_ktraj(*coords)
    A = ops.joint2operators(ops.espirit(S), nft)
    yt = torch.tensor(y.astype(np.complex64), device="cuda")
    xg, norms = solvers.cg_sense(A, yt, n_iter=8, use_graph=use_graph)
    x64 = _cg_fp64(coords, S, y, shape, 8)
    assert rel(xg.reshape(shape), x64) < 1e-3
    assert norms[-1] < norms[0]


def test_fista_haar_3d_matches_fp64_iterates():
    rng = np.random.default_rng(33)
    shape, nc = (16, 16, 16), 2
    kk = synth.centre_out_radial_3d(300, 16)
    dcf = np.maximum(np.sqrt(kk[0] ** 2 + kk[1] ** 2 + kk[2] ** 2), 1e-3) ** 2
    S = synth.coil_maps(shape, nc, rng)
    x = synth.ellipsoid_phantom(16, rng)
    op64 = O.NUFFT3dOracle(shape, dcf)
    op64.normalize_set_ktraj(np.stack(kk))
    y = op64.forward((x[..., None] * S).astype(np.complex128))

    nft = ops.NUFFT3d(shape, dcf)
    nft.normalize_set_ktraj(np.stack(kk))
    A = ops.joint2operators(ops.espirit(S), nft)
    W = solvers.DWTnd("haar", level=2, axes=(0, 1, 2))
    xg = solvers.FIST_wrap(A, W, torch.tensor(y.astype(np.complex64), device="cuda"), 4, 0.5, 1e-4)

    # FP64 restatement of the same FISTA with the oracle operators and the same wavelet
    class A64:
        def forward(self, v):
            return op64.forward(v * S)

        def backward(self, kd):
            return np.sum(np.conj(S) * op64.backward(kd), axis=-1, keepdims=True)

        def forward_backward(self, v):
            return np.sum(np.conj(S) * op64.forward_backward(v * S), axis=-1, keepdims=True)

    class W64:
        def forward(self, v):
            return SO.haar_idwt(v, 2, (0, 1, 2))

        def backward(self, v):
            return SO.haar_dwt(v, 2, (0, 1, 2))

    a, w = A64(), W64()
    invAb = a.backward(y)
    yv = 0.5 * invAb
    y_acc = np.zeros_like(yv)
    x_pre = yv
    t = [1.0] * 5
    for it in range(4):
        r = a.forward_backward(yv) - invAb
        y_acc = y_acc - 0.5 * r
        tf = w.backward(y_acc)
        aa = np.maximum(np.abs(tf) - 1e-4, 0)
        xx = w.forward(tf / (np.abs(tf) + 1e-6) * aa)
        t[it + 1] = (1 + (1 + 4 * t[it] ** 2) ** 0.5) / 2
        yv = xx + ((t[it] - 1) / t[it + 1]) * (xx - x_pre)
        x_pre = xx
    assert rel(xg, xx) < 1e-3


def test_ist_haar_3d_optscaled_matches_fp64_iterates():
    """The C4 solve's recipe at 32^3: data divided by optscaling (max |A^H y|,
    utilities/utilities_func.py:381-383) as examples/pics_IST_3dute_wavelet_L1.py:79-80 does,
    then IST_wrap with DWTnd('haar', 4), step 0.1, th 0.06; the GPU iterates follow the FP64
    restatement with the oracle operators (IST_32, CS_MRI_solvers_func.py:75-86)."""
    from mripy_gb300.utilities import optscaling
    rng = np.random.default_rng(34)
    n, nc, it = 32, 2, 10
    shape = (n, n, n)
    kk = synth.centre_out_radial_3d(1250, n)
    dcf = np.maximum(np.sqrt(kk[0] ** 2 + kk[1] ** 2 + kk[2] ** 2), 1e-3) ** 2
    dcf = dcf / dcf.mean()
    S = synth.coil_maps(shape, nc, rng)
    x = synth.ellipsoid_phantom(n, rng)
    op64 = O.NUFFT3dOracle(shape, dcf)
    op64.normalize_set_ktraj(np.stack(kk))
    y = op64.forward((x[..., None] * S).astype(np.complex128))
    y = y + 0.01 * np.abs(y).mean() * (rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape))

    nft = ops.NUFFT3d(shape, dcf)
    nft.normalize_set_ktraj(np.stack(kk))
    A = ops.joint2operators(ops.espirit(S), nft)
    yt = torch.tensor(y.astype(np.complex64), device="cuda")
    s_gpu = optscaling(A, yt)

    def back64(kd):
        return np.sum(np.conj(S) * op64.backward(kd), axis=-1, keepdims=True)

    def normal64(v):
        return np.sum(np.conj(S) * op64.forward_backward(v * S), axis=-1, keepdims=True)

    s64 = float(np.max(np.abs(back64(y))))
    assert abs(s_gpu - s64) / s64 < 1e-4
    W = solvers.DWTnd("haar", level=4, axes=(0, 1, 2))
    xg = solvers.IST_wrap(A, W, yt / s_gpu, it, 0.1, 0.06)
    x64 = SO.ist(normal64, back64(y / s64), it, 0.1, 0.06, 4, (0, 1, 2))
    assert rel(xg, x64) < 1e-3
