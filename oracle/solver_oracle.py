"""Oracle for the solver kernels: test infrastructure, never the product.

Only ``tests/`` may import this module, as the checker.  It restates in FP64 numpy:

* ``haar_dwt`` / ``haar_idwt``   DWTnd('haar', level, axes).backward / .forward
                                 (pics/operators_class.py:394-416 -> dwt/dwt_func.py:15-23:
                                 pywt.wavedecn + pywt.coeffs_to_array, and array_to_coeffs +
                                 waverecn).  pywt (PyWavelets) is not part of the reference
                                 tree and is not installed here; its published Haar analysis
                                 is restated: per axis a = (x[2k] + x[2k+1]) / sqrt(2),
                                 d = (x[2k] - x[2k+1]) / sqrt(2), applied to every axis at each
                                 level, the next level acting on the all-approximation block;
                                 coeffs_to_array puts the approximation first along every axis
                                 and each detail block at the slices its 'a'/'d' key names.
* ``soft_thresh``                prox_l1_soft_thresh2           pics/proximal_func.py:20-24
* ``prox_haar``                  prox_l1_Tf_soft_thresh2        pics/proximal_func.py:46-52
* ``ist`` / ``fista``            IST_32 / FIST_32               pics/CS_MRI_solvers_func.py:75-86, 207-224
                                 (the reference file is Python 2 syntax and cannot be imported)
* ``cg``                         linear CG on the normal equations, the algorithm of the
                                 commented-out block pics/proximal_func.py:379-406
* ``pipe_menon_dcf``             density compensation by Pipe-Menon iteration with the
                                 oracle's FP64 Gaussian spread/interp (gridding.c); the
                                 reference reads dcf from files (examples/
                                 pics_IST_3dute_wavelet_L1.py:31) and has no estimator

Parity of the Haar restatement is pinned by known answers of the published transform
(``tests/test_solver_oracle.py``): the level-2 Haar of [1..8] is [5, 13, -2, -2, -1/sqrt2 x 4],
and the 2-D / 3-D block layout of coeffs_to_array on hand-checked inputs.  The Pipe-Menon
restatement is pinned by its defining property: at the fixed point every sample's
gridded-and-interpolated weight is equal.
"""
import numpy as np

__all__ = ["haar_dwt", "haar_idwt", "soft_thresh", "prox_haar", "ist", "fista", "cg", "pipe_menon_dcf"]

_R2 = 1.0 / np.sqrt(2.0)


def _axes(x, axes):
    return tuple(int(a) % x.ndim for a in axes)


def haar_dwt(x, level, axes):
    """Image -> coefficient array (pywt.coeffs_to_array layout), FP64 complex."""
    y = np.array(x, dtype=np.complex128)
    axes = _axes(y, axes)
    n = [y.shape[a] for a in axes]
    for _ in range(level):
        if any(v % 2 for v in n):
            raise ValueError("axis sizes must be divisible by 2^level")
        sl = [slice(None)] * y.ndim
        for a, na in zip(axes, n):
            sl[a] = slice(0, na)
        blk = y[tuple(sl)].copy()
        for a in axes:
            e = np.take(blk, np.arange(0, blk.shape[a], 2), axis=a)
            o = np.take(blk, np.arange(1, blk.shape[a], 2), axis=a)
            blk = np.concatenate([(e + o) * _R2, (e - o) * _R2], axis=a)
        y[tuple(sl)] = blk
        n = [v // 2 for v in n]
    return y


def haar_idwt(c, level, axes):
    """Coefficient array -> image, the inverse of ``haar_dwt``."""
    y = np.array(c, dtype=np.complex128)
    axes = _axes(y, axes)
    full = [y.shape[a] for a in axes]
    for lv in reversed(range(level)):
        n = [v >> lv for v in full]
        sl = [slice(None)] * y.ndim
        for a, na in zip(axes, n):
            sl[a] = slice(0, na)
        blk = y[tuple(sl)].copy()
        for a, na in zip(axes, n):
            h = na // 2
            lo = np.take(blk, np.arange(0, h), axis=a)
            hi = np.take(blk, np.arange(h, na), axis=a)
            e, o = (lo + hi) * _R2, (lo - hi) * _R2
            out = np.empty_like(blk)
            idx = [slice(None)] * blk.ndim
            idx[a] = slice(0, na, 2)
            out[tuple(idx)] = e
            idx[a] = slice(1, na, 2)
            out[tuple(idx)] = o
            blk = out
        y[tuple(sl)] = blk
    return y


def soft_thresh(x, th):
    a = np.abs(x)
    return x / (a + 1e-6) * np.maximum(a - th, 0.0)


def prox_haar(x, th, level, axes):
    return haar_idwt(soft_thresh(haar_dwt(x, level, axes), th), level, axes)


def ist(normal, rhs, n_iter, step, th, level, axes):
    """IST_32 with invAAfunc = normal and invAb = rhs."""
    x_acc = step * rhs
    x = x_acc
    for _ in range(n_iter):
        x = prox_haar(x_acc, th, level, axes)
        r = normal(x) - rhs
        x_acc = x_acc - step * r
    return x


def fista(normal, rhs, n_iter, step, th, level, axes):
    """FIST_32 with invAAfunc = normal and invAb = rhs."""
    y = step * rhs
    y_acc = np.zeros_like(y)
    x_pre = y
    t = np.ones(n_iter + 1)
    x = y
    for k in range(n_iter):
        r = normal(y) - rhs
        y_acc = y_acc - step * r
        x = prox_haar(y_acc, th, level, axes)
        t[k + 1] = (1 + (1 + 4 * t[k] ** 2) ** 0.5) / 2
        y = x + ((t[k] - 1) / t[k + 1]) * (x - x_pre)
        x_pre = x
    return x


def pipe_menon_dcf(coords, shape, n_iter, eps=1e-5, offsets=None):
    """Pipe-Menon density compensation (J. G. Pipe, P. Menon, MRM 41:179, 1999) with the
    Gaussian gridding kernel of the NUFFT at ``eps``: w = 1, w <- w / |interp(spread(w))|,
    then w scaled to mean 1 in every trajectory group (``offsets``: group boundaries)."""
    from . import nufft_oracle as NO
    dim = len(shape)
    ns, nf, tau = NO._params_for(dim, tuple(shape), eps)
    xs = [np.asarray(v, dtype=np.float64) for v in coords]
    M = len(xs[0])
    offsets = [0, M] if offsets is None else list(offsets)
    w = np.ones(M)
    for _ in range(n_iter):
        cw = np.ones(M, dtype=np.complex128)
        for a, b in zip(offsets[:-1], offsets[1:]):
            if b == a:
                continue
            sub = [v[a:b] for v in xs]
            G = NO.spread(sub, w[None, a:b].astype(np.complex128), tau, ns, nf)
            cw[a:b] = NO.interp(sub, G, tau, ns)[0]
        w = w / np.abs(cw)
    for a, b in zip(offsets[:-1], offsets[1:]):
        if b > a:
            w[a:b] *= (b - a) / w[a:b].sum()
    return w


def cg(normal, rhs, n_iter, x0=None):
    """Linear CG on normal(x) = rhs; returns (x, residual norms after every iteration)."""
    x = np.zeros_like(rhs) if x0 is None else np.array(x0, dtype=rhs.dtype)
    r = rhs - normal(x) if x0 is not None else rhs.copy()
    p = r.copy()
    rs = np.vdot(r, r).real
    norms = []
    for _ in range(n_iter):
        q = normal(p)
        a = rs / np.vdot(p, q).real
        x = x + a * p
        r = r - a * q
        rn = np.vdot(r, r).real
        p = r + (rn / rs) * p
        rs = rn
        norms.append(np.sqrt(rn))
    return x, np.array(norms)
