"""Drop-in NUFFT functions with the signatures of mripy's ``fft/nufft_func.py`` and
``fft/nufft_func_cuda.py``, computed by the GB300 library.

Inputs may be numpy arrays (uploaded once; the result comes back as numpy in the
input's complex precision, complex128 for the reference's usual float64/complex128
inputs) or torch CUDA tensors (zero-copy; the result is a complex64 CUDA tensor).
Arithmetic is complex64 on the GPU; eps selects nspread/oversampling/tau exactly as
the reference does.  ``gridfast`` and ``save_ram`` are accepted and ignored (there is
one GPU path).  Trailing dimensions after the sample axis (type-1 input, type-2
output) or after the image axes (type-2 input, type-1 output) are coils, as in the
reference (``utilities_func.dim_match``); unlike the reference's 2-D type-2
(which allocates its output as ``np.zeros(x.shape)``, nufft_func.py:612) every
function here accepts them.
"""
from collections import OrderedDict

import numpy as np
import torch

from .plan import NufftPlan, grid_params

__all__ = [
    "_compute_1d_grid_params", "_compute_2d_grid_params", "_compute_3d_grid_params",
    "nufftfreqs1d", "nufftfreqs2d", "nufftfreqs3d",
    "nufft1d1_gaussker", "nufft1d2_gaussker", "nufft1d21_gaussker",
    "nufft2d1_gaussker", "nufft2d2_gaussker", "nufft2d21_gaussker",
    "nufft3d1_gaussker", "nufft3d2_gaussker", "nufft3d21_gaussker",
    "nufft1d1_gaussker_cuda", "nufft1d2_gaussker_cuda", "nufft1d21_gaussker_cuda",
    "nufft2d1_gaussker_cuda", "nufft2d2_gaussker_cuda", "nufft2d21_gaussker_cuda",
    "nufft3d1_gaussker_cuda", "nufft3d2_gaussker_cuda", "nufft3d21_gaussker_cuda",
    "clear_plan_cache",
]


# ---------------------------------------------------------------- parameters (nufft_func.py:198-249)
def _compute_1d_grid_params(ms, eps):
    ns, nf, tau = grid_params(1, ms, 1, 1, eps)
    return ns, nf[0], tau


def _compute_2d_grid_params(ms, mt, eps):
    ns, nf, tau = grid_params(2, ms, mt, 1, eps)
    return ns, nf[0], nf[1], tau


def _compute_3d_grid_params(ms, mt, mu, eps, max_nspread=None):
    ns, nf, tau = grid_params(3, ms, mt, mu, eps, max_nspread or 0)
    return ns, nf[0], nf[1], nf[2], tau


# ---------------------------------------------------------------- frequencies (nufft_func.py:59-167)
def nufftfreqs1d(ms, df=1):
    return df * np.arange(-(ms // 2), ms - (ms // 2))


def nufftfreqs2d(ms, mt, df=1.0):
    return df * np.mgrid[-(ms // 2): ms - (ms // 2), -(mt // 2): mt - (mt // 2)]


def nufftfreqs3d(ms, mt, mu, df=1.0):
    return df * np.mgrid[-(ms // 2): ms - (ms // 2), -(mt // 2): mt - (mt // 2), -(mu // 2): mu - (mu // 2)]


# ---------------------------------------------------------------- plan cache
_PLANS = OrderedDict()
_MAX_PLANS = 8


def clear_plan_cache():
    for p in _PLANS.values():
        p.close()
    _PLANS.clear()


def _plan(dim, shape, n_coil, eps, iflag, df, max_nspread):
    key = (dim, tuple(shape), n_coil, float(eps), 1 if iflag >= 0 else -1, float(df), max_nspread)
    p = _PLANS.get(key)
    if p is None:
        p = NufftPlan(dim, shape, n_coil=n_coil, n_traj=1, eps=eps, iflag=iflag, df=df, max_nspread=max_nspread)
        _PLANS[key] = p
        while len(_PLANS) > _MAX_PLANS:
            _PLANS.popitem(last=False)[1].close()
    else:
        _PLANS.move_to_end(key)
    return p


def _coords(arrs):
    out = []
    for a in arrs:
        if isinstance(a, torch.Tensor):
            t = a.detach()
            if t.dtype not in (torch.float32, torch.float64):
                t = t.to(torch.float64)
            out.append(t.to("cuda").reshape(-1))
        else:
            out.append(torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))).to("cuda"))
    dt = torch.float64 if any(t.dtype == torch.float64 for t in out) else torch.float32
    return [t.to(dt) for t in out]


def _data(a):
    """(complex64 CUDA tensor, was_numpy, numpy result dtype)"""
    if isinstance(a, torch.Tensor):
        t = a.detach().to("cuda")
        if t.dtype != torch.complex64:
            t = t.to(torch.complex64)
        return t, False, None
    arr = np.asarray(a)
    res = np.complex64 if arr.dtype in (np.complex64, np.float32) else np.complex128
    return torch.from_numpy(np.ascontiguousarray(arr.astype(np.complex64))).to("cuda"), True, res


def _back(t, was_numpy, res):
    return t.cpu().numpy().astype(res) if was_numpy else t


def _weights(dcf, M):
    if dcf is None:
        return None
    if isinstance(dcf, torch.Tensor):
        w = dcf.detach().to("cuda", torch.float32).reshape(-1).contiguous()
    else:
        w = torch.from_numpy(np.ascontiguousarray(np.asarray(dcf, dtype=np.float32).reshape(-1))).to("cuda")
    if w.numel() != M:
        raise ValueError("dcf must have one entry per sample")
    return w


def _type1(coords, c, shape, df, eps, iflag, max_nspread):
    ct, was_np, res = _data(c)
    M = ct.shape[0]
    trail = tuple(ct.shape[1:])
    nc = int(np.prod(trail)) if trail else 1
    p = _plan(len(shape), shape, nc, eps, iflag, df, max_nspread)
    p.set_points(_coords(coords))
    out = p.type1(ct.reshape(M, nc))
    return _back(out.reshape(tuple(shape) + trail), was_np, res)


def _type2(coords, Fk, shape, df, eps, iflag, max_nspread):
    ft, was_np, res = _data(Fk)
    dim = len(shape)
    trail = tuple(ft.shape[dim:])
    nc = int(np.prod(trail)) if trail else 1
    p = _plan(dim, shape, nc, eps, iflag, df, max_nspread)
    p.set_points(_coords(coords))
    out = p.type2(ft.reshape((1,) + tuple(shape) + (nc,)))
    return _back(out.reshape((p.n_samples,) + trail), was_np, res)


def _type21(coords, Fk, shape, df, eps, iflag, max_nspread, dcf=None):
    ft, was_np, res = _data(Fk)
    dim = len(shape)
    trail = tuple(ft.shape[dim:])
    nc = int(np.prod(trail)) if trail else 1
    p = _plan(dim, shape, nc, eps, iflag, df, max_nspread)
    p.set_points(_coords(coords))
    out = p.type21(ft.reshape((1,) + tuple(shape) + (nc,)), dcf=_weights(dcf, p.n_samples))
    return _back(out.reshape(tuple(shape) + trail), was_np, res)


# ---------------------------------------------------------------- 1-D (nufft_func.py:438-545)
def nufft1d1_gaussker(x, c, ms, df=1.0, eps=1E-15, iflag=1, gridfast=1):
    return _type1((x,), c, (ms,), df, eps, iflag, None)


def nufft1d2_gaussker(x, Fk, ms, df=1.0, eps=1E-15, iflag=1, gridfast=1):
    return _type2((x,), Fk, (ms,), df, eps, iflag, None)


def nufft1d21_gaussker(x, Fk, ms, df=1.0, eps=1E-15, iflag=1, gridfast=0):
    return _type21((x,), Fk, (ms,), df, eps, iflag, None)


# ---------------------------------------------------------------- 2-D (nufft_func.py:702-830)
def nufft2d1_gaussker(x, y, c, ms, mt, df=1.0, eps=1E-15, iflag=1, gridfast=1):
    return _type1((x, y), c, (ms, mt), df, eps, iflag, None)


def nufft2d2_gaussker(x, y, Fk, ms, mt, df=1.0, eps=1E-15, iflag=1, gridfast=1):
    return _type2((x, y), Fk, (ms, mt), df, eps, iflag, None)


def nufft2d21_gaussker(x, y, Fk, ms, mt, df=1.0, eps=1E-15, iflag=1, gridfast=1):
    return _type21((x, y), Fk, (ms, mt), df, eps, iflag, None)


# ---------------------------------------------------------------- 3-D (nufft_func.py:1167-1330)
def nufft3d1_gaussker(x, y, z, c, ms, mt, mu, df=1.0, eps=1E-15, iflag=1, gridfast=1):
    return _type1((x, y, z), c, (ms, mt, mu), df, eps, iflag, 6)


def nufft3d2_gaussker(x, y, z, Fk, ms, mt, mu, df=1.0, eps=1E-15, iflag=1, gridfast=0):
    return _type2((x, y, z), Fk, (ms, mt, mu), df, eps, iflag, 6)


def nufft3d21_gaussker(x, y, z, Fk, ms, mt, mu, dcf=None, df=1.0, eps=1E-15, iflag=1, gridfast=0):
    return _type21((x, y, z), Fk, (ms, mt, mu), df, eps, iflag, 6, dcf)


# ---------------------------------------------------------------- _cuda twins (nufft_func_cuda.py)
def nufft1d1_gaussker_cuda(x, c, ms, df=1.0, eps=1E-15, iflag=1, gridfast=1):
    return nufft1d1_gaussker(x, c, ms, df, eps, iflag)


def nufft1d2_gaussker_cuda(x, Fk, ms, df=1.0, eps=1E-15, iflag=1, gridfast=1):
    return nufft1d2_gaussker(x, Fk, ms, df, eps, iflag)


def nufft1d21_gaussker_cuda(x, Fk, ms, df=1.0, eps=1E-15, iflag=1, gridfast=0):
    return nufft1d21_gaussker(x, Fk, ms, df, eps, iflag)


def nufft2d1_gaussker_cuda(x, y, c, ms, mt, df=1.0, eps=1E-15, iflag=1, gridfast=1):
    return nufft2d1_gaussker(x, y, c, ms, mt, df, eps, iflag)


def nufft2d2_gaussker_cuda(x, y, Fk, ms, mt, df=1.0, eps=1E-15, iflag=1, gridfast=0):
    return nufft2d2_gaussker(x, y, Fk, ms, mt, df, eps, iflag)


def nufft2d21_gaussker_cuda(x, y, Fk, ms, mt, df=1.0, eps=1E-15, iflag=1, gridfast=0):
    return nufft2d21_gaussker(x, y, Fk, ms, mt, df, eps, iflag)


def nufft3d1_gaussker_cuda(x, y, z, c, ms, mt, mu, df=1.0, eps=1E-15, iflag=1, gridfast=1, save_ram=1):
    return nufft3d1_gaussker(x, y, z, c, ms, mt, mu, df, eps, iflag)


def nufft3d2_gaussker_cuda(x, y, z, Fk, ms, mt, mu, df=1.0, eps=1E-15, iflag=1, gridfast=1, save_ram=0):
    return nufft3d2_gaussker(x, y, z, Fk, ms, mt, mu, df, eps, iflag)


def nufft3d21_gaussker_cuda(x, y, z, Fk, ms, mt, mu, dcf, df=1.0, eps=1E-15, iflag=1, gridfast=0, save_ram=1):
    return nufft3d21_gaussker(x, y, z, Fk, ms, mt, mu, dcf, df, eps, iflag)
