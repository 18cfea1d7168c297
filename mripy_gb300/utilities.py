"""Data scaling helpers that mripy's reconstruction scripts apply before a solver
(utilities/utilities_func.py:378-388).

* ``optscaling(FT, b)``  the largest magnitude of ``FT.backward(b)``: dividing the k-space
                         data by it puts the adjoint image's peak at 1, so a solver
                         threshold (IST/FISTA's ``th``) is relative to the image's scale.
* ``scaling(b)``         the largest element of ``b`` (mripy takes ``max`` of the array
                         itself, which for complex data orders by real part; the same here).
"""
import numpy as np
import torch


def optscaling(FT, b):
    """max |FT.backward(b)| as a Python float (utilities_func.py:381-383)."""
    x0 = FT.backward(b)
    if isinstance(x0, torch.Tensor):
        return float(torch.max(torch.abs(x0)))
    return float(np.max(np.absolute(np.asarray(x0)).flatten()))


def scaling(b):
    """max(b.flatten()) (utilities_func.py:387-388)."""
    if isinstance(b, torch.Tensor):
        b = b.detach().cpu().numpy()
    flat = np.asarray(b).flatten()
    if np.iscomplexobj(flat):
        # numpy orders complex numbers lexicographically (real part, then imaginary)
        return flat[np.lexsort((flat.imag, flat.real))[-1]]
    return flat.max()


def universal_threshold(im, axes=None):
    """Wavelet soft threshold from the data's own noise level: Donoho and Johnstone's
    universal threshold sigma * sqrt(2 ln N) (Biometrika 81:425, 1994), with sigma the
    median absolute finest-scale diagonal Haar detail coefficient / 0.6745 (over real and
    imaginary parts) and N the pixel count.  For an IST/FISTA solve on data scaled by
    ``optscaling``, ``im`` is the scaled adjoint image; the result is used as ``th``.
    mripy takes ``th`` as a fixed number (examples/pics_IST_3dute_wavelet_L1.py:94); this
    helper only chooses one for data whose noise level differs from that example's."""
    from .solvers import DWTnd
    t = im if isinstance(im, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(np.asarray(im)))
    t = t.to("cuda", torch.complex64)
    axes = tuple(range(min(t.dim(), 3))) if axes is None else tuple(axes)
    c = DWTnd("haar", level=1, axes=axes).backward(t)
    sl = [slice(None)] * c.dim()
    for a in axes:
        sl[a] = slice(c.shape[a] // 2, None)
    d = c[tuple(sl)].reshape(-1)
    parts = torch.cat([d.real, d.imag]).abs()
    sigma = float(parts.median()) / 0.6745
    n = 1
    for a in axes:
        n *= int(t.shape[a])
    return sigma * float(np.sqrt(2.0 * np.log(n)))
