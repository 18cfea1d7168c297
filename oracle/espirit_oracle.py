"""Oracle for ESPIRiT coil maps: test infrastructure, never the product.

Only ``tests/`` may import this module, as the checker.  It restates in FP64 numpy
``espirit_2d`` / ``espirit_3d`` (espirit/espirit_func.py:25-95, 110-219) and the helpers
they call:

* ``hankel_matrix``   hankelnd_r (pics/hankel_func.py:190-207) with the window (w..., 1)
                      and the reshape of espirit_func.py:36-41 / 130-135: rows = positions
                      inside the window, columns = window movements x coils
* ``hamming_nd``      hamming2d / hamming3d (signal_processing/filter_func.py:30-40):
                      sqrt, resp. cube root, of the outer product of symmetric Hamming
                      windows 0.54 - 0.46 cos(2 pi n / (M - 1)) (scipy.signal.hamming)
* ``pad_center``      pad2d / pad3d (utilities/utilities_func.py:288-309, 359-376): the data
                      at [n//2 - d//2, ...) of a zero array
* ``ft_forward``, ``ft_backward``   FFTW2d / FFTWnd (pics/operators_class.py:169-187):
                      fftshift, FFT (pyFFTW's inverse is normalised as numpy.fft.ifftn),
                      ifftshift
* ``espirit``         the whole function

The reference does not run as written on Python 3 with numpy 2 (np.int, map objects inside
np.ix_), and espirit_2d's threshold reads ``nsing_th``, which is undefined; the restatement
follows espirit_3d's ``nsigv_th`` in both.  Kept as in the reference: the kept count is the LAST
index k with s[k] > s[0] * nsigv_th (so one fewer than the singular values above it).
Deviation: the eigenvector phase is canonical (the first coil with a non-zero component
made real and non-negative) where the reference keeps LAPACK's arbitrary per-pixel phase.
Parity is pinned against the reference's own outputs (``tests/golden/golden_espirit.npz``,
made by ``tests/golden/make_golden_solvers.py`` from espirit_func.py itself): the
eigenvalue maps agree to rounding, and the coil maps agree up to one phase per pixel
wherever no FFT resampling follows the eigen step (resampling maps of arbitrary per-pixel
phase, as the reference does with pad_before_espirit = 0 and a smaller calibration grid,
gives phase-dependent values there).  ``tests/test_espirit_oracle.py`` also checks the
recovery of known coil maps.
"""
import numpy as np

__all__ = ["hankel_matrix", "hamming_nd", "pad_center", "ft_forward", "ft_backward", "kept_count",
           "eigen_pixels", "espirit"]


def hankel_matrix(xcrop, win):
    """(prod(win), prod(moves) * nc) matrix of a[i + m, c] for window position i, move m."""
    d = len(win)
    a = np.asarray(xcrop)
    moves = tuple(a.shape[k] - win[k] + 1 for k in range(d))
    nc = a.shape[d]
    out = np.empty((int(np.prod(win)),) + moves + (nc,), dtype=np.complex128)
    for idx, i in enumerate(np.ndindex(*win)):
        sl = tuple(slice(i[k], i[k] + moves[k]) for k in range(d))
        out[idx] = a[sl]
    return out.reshape(out.shape[0], -1), moves


def _hamming(n):
    if n == 1:
        return np.ones(1)
    k = np.arange(n)
    return 0.54 - 0.46 * np.cos(2 * np.pi * k / (n - 1))


def hamming_nd(shape):
    w = _hamming(shape[0])
    for n in shape[1:]:
        w = np.multiply.outer(w, _hamming(n))
    return w ** (1.0 / len(shape))


def pad_center(data, sizes):
    out = np.zeros(tuple(sizes) + data.shape[len(sizes):], dtype=data.dtype)
    sl = tuple(slice(n // 2 - d // 2, n // 2 - d // 2 + d) for n, d in zip(sizes, data.shape))
    out[sl] = data
    return out


def ft_forward(x, axes):
    return np.fft.ifftshift(np.fft.fftn(np.fft.fftshift(x, axes), axes=axes), axes)


def ft_backward(x, axes):
    return np.fft.ifftshift(np.fft.ifftn(np.fft.fftshift(x, axes), axes=axes), axes)


def kept_count(s, nsigv_th, nsingularv=150):
    for k in range(len(s)):
        if s[k] > s[0] * nsigv_th:
            nsingularv = k
    return nsingularv


def eigen_pixels(imvn):
    """imvn (..., nsv, nc): per pixel the top eigenpair of vvH = A^T conj(A)."""
    sh = imvn.shape[:-2]
    nc = imvn.shape[-1]
    A = imvn.reshape((-1,) + imvn.shape[-2:])
    vvH = np.einsum("pkc,pkd->pcd", A, np.conj(A))
    lam, vec = np.linalg.eigh(vvH)
    v = vec[:, :, -1]
    s = lam[:, -1]
    for p in range(v.shape[0]):
        nz = np.nonzero(np.abs(v[p]) > 0)[0]
        if len(nz):
            v[p] *= np.conj(v[p, nz[0]]) / np.abs(v[p, nz[0]])
    return v.reshape(sh + (nc,)), s.reshape(sh)


def espirit(xcrop, x_shape, nsingularv=150, hkwin_shape=(16, 16), pad_before_espirit=0, pad_fact=1,
            sigv_th=0.01, nsigv_th=0.2, return_info=False):
    d = len(hkwin_shape)
    axes = tuple(range(d))
    xcrop = np.asarray(xcrop, dtype=np.complex128)
    hmtx, moves = hankel_matrix(xcrop, tuple(hkwin_shape))
    _, s, V = np.linalg.svd(hmtx, full_matrices=False)
    nsv = kept_count(s, nsigv_th, nsingularv)
    nc = x_shape[d]
    vn = V[:nsv].reshape((nsv,) + moves + (nc,))
    vn = np.moveaxis(vn, 0, d)                               # moves + (nsv, nc)
    if pad_before_espirit == 0:
        n = tuple(min(pad_fact * xcrop.shape[k], x_shape[k]) for k in range(d))
    else:
        n = tuple(x_shape[:d])
    vn = vn * hamming_nd(moves)[(...,) + (None,) * 2]
    imvn = ft_backward(pad_center(vn, n), axes)
    Vim, sim = eigen_pixels(imvn)
    sim = sim.astype(np.complex128)
    if pad_before_espirit == 0:
        Vim = ft_backward(pad_center(ft_forward(Vim, axes), x_shape[:d]), axes)
        sim = ft_backward(pad_center(ft_forward(sim, axes), x_shape[:d]), axes)
    Vim = Vim / (1e-6 + np.linalg.norm(Vim, axis=d))[..., None]
    sim = normalise_eigenvalues(sim)
    Vim[np.real(sim) < sigv_th] = 0
    if return_info:
        return Vim, np.abs(sim), {"nsv": nsv, "singular_values": s}
    return Vim, np.abs(sim)


def normalise_eigenvalues(sim):
    """sim / max(sim) as espirit_func.py:95 / 212 evaluates it on the complex map: numpy
    orders complex numbers by real part (then imaginary part), so the divisor is the
    element of largest real part, imaginary part and all; the threshold that follows
    (sim < sigv_th) compares real parts the same way."""
    flat = np.asarray(sim, dtype=np.complex128).reshape(-1)
    return sim / flat[np.lexsort((flat.imag, flat.real))[-1]]
