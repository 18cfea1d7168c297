"""ESPIRiT coil-sensitivity maps on the GPU: ``espirit_2d`` / ``espirit_3d`` with the
signatures and defaults of espirit/espirit_func.py:25, 110.

Steps (the reference's, on device tensors):
1. block-Hankel matrix of the calibration k-space (hankelnd_r, pics/hankel_func.py:190-207,
   window (w..., 1)): rows = positions inside the window, columns = window moves x coils;
2. its SVD (cuSOLVER through torch.linalg.svd, a library call), keeping the first k rows of
   V^H with k the last index whose singular value exceeds nsigv_th * s[0];
3. the kept rows as k-space kernels (moves x coils), times the Hamming window
   (hamming2d / hamming3d), zero-padded to the map grid and brought to image space with the
   reference's shifted inverse FFT (cuFFT);
4. per pixel the top eigenpair of vvH = A^T conj(A) -- the library's ``gbn_espirit_eigen``
   kernel (one warp per pixel, power iterations);
5. with pad_before_espirit == 0, maps and eigenvalues resampled to x_shape by FFT padding;
   maps normalised per pixel, pixels whose normalised eigenvalue is below sigv_th zeroed.

As written the reference's espirit_2d reads an undefined name (``nsing_th``) in step 2;
both functions here use ``nsigv_th`` as espirit_3d does.  The eigenvector phase per pixel
is fixed (first non-zero coil real and non-negative) where the reference keeps LAPACK's
arbitrary phase; after resampling the eigenvalue map's real part is normalised.
numpy in -> numpy out (complex128 maps); torch CUDA in -> torch CUDA out.
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from .plan import _stream

__all__ = ["espirit_2d", "espirit_3d", "espirit_nd", "espirit_eigen"]


def _hamming(n):
    if n == 1:
        return np.ones(1)
    k = np.arange(n)
    return 0.54 - 0.46 * np.cos(2 * np.pi * k / (n - 1))


def _window(moves):
    w = _hamming(moves[0])
    for n in moves[1:]:
        w = np.multiply.outer(w, _hamming(n))
    return w ** (1.0 / len(moves))


def _pad_center(t, sizes):
    d = len(sizes)
    out = torch.zeros(tuple(sizes) + tuple(t.shape[d:]), dtype=t.dtype, device=t.device)
    sl = tuple(slice(n // 2 - m // 2, n // 2 - m // 2 + m) for n, m in zip(sizes, t.shape[:d]))
    out[sl] = t
    return out


def _ft_forward(t, dims):
    return torch.fft.ifftshift(torch.fft.fftn(torch.fft.fftshift(t, dims), dim=dims), dims)


def _ft_backward(t, dims):
    return torch.fft.ifftshift(torch.fft.ifftn(torch.fft.fftshift(t, dims), dim=dims), dims)


def espirit_eigen(a, n_iter=64, stream=None):
    """a: (..., nsv, nc) complex64 CUDA tensor of image-space kernels -> (maps (..., nc),
    eigenvalues (...)): the top eigenpair of A^T conj(A) per pixel."""
    if not (isinstance(a, torch.Tensor) and a.is_cuda and a.dtype == torch.complex64):
        raise TypeError("a must be a complex64 CUDA tensor")
    a = a.contiguous()
    lead = tuple(a.shape[:-2])
    nsv, nc = int(a.shape[-2]), int(a.shape[-1])
    n_pix = int(np.prod(lead)) if lead else 1
    vmap = torch.empty(lead + (nc,), dtype=torch.complex64, device=a.device)
    smap = torch.empty(lead, dtype=torch.float32, device=a.device)
    N.check(N.lib().gbn_espirit_eigen(ctypes.c_void_p(a.data_ptr()), n_pix, nsv, nc, int(n_iter),
                                      ctypes.c_void_p(vmap.data_ptr()), ctypes.c_void_p(smap.data_ptr()),
                                      _stream(stream)))
    return vmap, smap


def espirit_nd(xcrop, x_shape, nsingularv=150, hkwin_shape=(16, 16), pad_before_espirit=0, pad_fact=1,
               sigv_th=0.01, nsigv_th=0.2, n_power_iter=64, return_info=False):
    """ESPIRiT over len(hkwin_shape) spatial axes; xcrop (calibration k-space, spatial axes
    then coils), x_shape = map shape + (nc,)."""
    d = len(hkwin_shape)
    was_np = not isinstance(xcrop, torch.Tensor)
    a = (torch.from_numpy(np.ascontiguousarray(np.asarray(xcrop).astype(np.complex64))).cuda() if was_np
         else xcrop.to("cuda", torch.complex64).contiguous())
    win = tuple(int(w) for w in hkwin_shape)
    moves = tuple(int(a.shape[k]) - win[k] + 1 for k in range(d))
    if any(m < 1 for m in moves):
        raise ValueError("the calibration region must be at least the window size")
    nc = int(a.shape[d])
    st = a.stride()
    view = torch.as_strided(a, win + moves + (nc,), st[:d] + st[:d] + (st[d],))
    hmtx = view.reshape(int(np.prod(win)), -1)
    r, ncol = int(hmtx.shape[0]), int(hmtx.shape[1])
    gram = r <= ncol
    if gram:
        # wide Hankel matrices: singular values and right vectors from the Gram matrix H H^H
        # and its FP64 eigendecomposition, 2-2.5x faster than the SVD on GB300.  The product
        # is FP64 up to r^2 c = 2^30 (2-D calibrations), FP32 beyond (3-D), where it blurs only
        # singular values far below the kept ones; the kept vectors v_k = U_k^H H / s_k have
        # s_k >= nsigv_th * s_0, and the maps depend on their span alone
        h = hmtx.to(torch.complex128) if r * r * ncol <= (1 << 30) else hmtx
        lam, U = torch.linalg.eigh((h @ h.conj().T).to(torch.complex128))
        s = lam.flip(0).clamp_min(0.0).sqrt()
        U = U.flip(1)
    else:
        _, s, vh = torch.linalg.svd(hmtx, full_matrices=False)
    s_host = s.cpu().numpy()
    nsv = nsingularv
    for k in range(len(s_host)):
        if s_host[k] > s_host[0] * nsigv_th:
            nsv = k
    if gram:
        vh = ((U[:, :nsv].conj().T.to(h.dtype) @ h) / s[:nsv, None].to(h.real.dtype)).to(torch.complex64)
    if pad_before_espirit == 0:
        n = tuple(min(pad_fact * int(a.shape[k]), int(x_shape[k])) for k in range(d))
    else:
        n = tuple(int(v) for v in x_shape[:d])
    dims = tuple(range(d))
    vn = vh[:nsv].reshape((nsv,) + moves + (nc,)).movedim(0, d)
    w = torch.from_numpy(_window(moves).astype(np.float32)).cuda()
    vn = vn * w.reshape(moves + (1, 1))
    imvn = _ft_backward(_pad_center(vn, n), dims).to(torch.complex64)
    vim, sim = espirit_eigen(imvn, n_power_iter)
    sim = sim.to(torch.complex64)
    if pad_before_espirit == 0:
        full = tuple(int(v) for v in x_shape[:d])
        vim = _ft_backward(_pad_center(_ft_forward(vim, dims), full), dims)
        sim = _ft_backward(_pad_center(_ft_forward(sim, dims), full), dims)
    vim = vim / (1e-6 + torch.linalg.vector_norm(vim, dim=d, keepdim=True))
    # sim / max(sim) on the complex map as numpy evaluates it (espirit_func.py:95, 212):
    # the divisor is the element of largest real part; the threshold compares real parts
    flat = sim.reshape(-1)
    sim = sim / flat[torch.argmax(flat.real)]
    vim = torch.where((sim.real < sigv_th)[..., None], torch.zeros((), dtype=vim.dtype, device=vim.device), vim)
    sim = sim.abs()
    if was_np:
        vim, sim = vim.cpu().numpy().astype(np.complex128), sim.cpu().numpy().astype(np.float64)
    if return_info:
        return vim, sim, {"nsv": nsv, "singular_values": s_host}
    return vim, sim


def espirit_2d(xcrop, x_shape, nsingularv=150, hkwin_shape=(16, 16), pad_before_espirit=0, pad_fact=1,
               sigv_th=0.01, nsigv_th=0.2):
    """espirit/espirit_func.py:25 -> (Vim (nx, ny, nc) coil maps, sim (nx, ny))."""
    return espirit_nd(xcrop, x_shape, nsingularv, hkwin_shape, pad_before_espirit, pad_fact, sigv_th, nsigv_th)


def espirit_3d(xcrop, x_shape, nsingularv=150, hkwin_shape=(16, 16, 16), pad_before_espirit=0, pad_fact=1,
               sigv_th=0.01, nsigv_th=0.2):
    """espirit/espirit_func.py:110 -> (Vim (nx, ny, nz, nc) coil maps, sim (nx, ny, nz))."""
    return espirit_nd(xcrop, x_shape, nsingularv, hkwin_shape, pad_before_espirit, pad_fact, sigv_th, nsigv_th)
