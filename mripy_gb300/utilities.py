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
