"""Oracle for the Gaussian-gridding NUFFT: test infrastructure, never the product.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module, and only as the checker or as the timed
CPU reference.  The GPU library never calls it.

It restates mripy's CPU NUFFT (peng-cao/mripy ``fft/nufft_func.py``) in FP64:

* ``grid_params``            ``_compute_{1,2,3}d_grid_params``  nufft_func.py:198-249
* ``freqs``                  ``nufftfreqs{1,2,3}d``             nufft_func.py:59-61, 104-106, 162-167
* ``nufft_type1``            ``nufft{1,2,3}d1_gaussker``        nufft_func.py:438-467, 702-738, 1167-1206
* ``nufft_type2``            ``nufft{1,2,3}d2_gaussker``        nufft_func.py:470-503, 741-777, 1209-1258
* ``nufft_type21``           ``nufft{1,2,3}d21_gaussker``       nufft_func.py:506-545, 780-830, 1261-1330
* ``NUFFT3dOracle``          ``NUFFT3d``                        pics/operators_class.py:302-364
* ``nudft_type1``            ``nudft{1,2,3}d1``                 nufft_func.py:41-45, 82-90, 138-146

The tap loops (spread/interp/normal) run in ``gridding.c`` (FP64, OpenMP over
coils) through ctypes; the FFT stage uses ``numpy.fft`` (or ``scipy.fft`` with
worker threads for the timed baseline), standing in for numpy/pyFFTW.  Parity
is pinned against golden vectors generated from the reference itself
(``tests/golden/make_golden.py``).

Trailing dimensions after the sample axis (type-1 input, type-2 output) and
after the image axes (type-2 input, type-1 output) are coils, as in the
reference (``utilities_func.dim_match``).
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None
_lock = threading.Lock()


def build(force=False):
    """Compile gridding.c into oracle/_build/liboracle.so (gcc, portable flags)."""
    src = os.path.join(_HERE, "gridding.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = ctypes.CDLL(_LIB_PATH)
    return _lib


_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp) if a is not None else None


# ---------------------------------------------------------------- parameters

def grid_params(dim, ms, mt=None, mu=None, eps=1e-15, max_nspread=None):
    """(nspread, nf tuple, tau) exactly as _compute_{1,2,3}d_grid_params (nufft_func.py:198-249)."""
    if eps <= 1e-33 or eps >= 1e-1:
        raise ValueError("eps = {0:.0e}; must satisfy 1e-33 < eps < 1e-1.".format(eps))
    rat = 2 if eps > 1e-11 else 3
    nspread = int(-np.log(eps) / (np.pi * (rat - 1) / (rat - 0.5)) + 0.5)
    if max_nspread is not None:
        nspread = min(nspread, max_nspread)
        nspread = max(nspread, 3)
    sizes = [ms, mt, mu][:dim]
    nf = tuple(max(rat * m, 2 * nspread) for m in sizes)
    lambda_ = nspread / (rat * (rat - 0.5))
    tau = np.pi * lambda_ / ms ** 2          # ms only, also for mt/mu (reference behaviour)
    return nspread, nf, tau


def freqs(m, df=1.0):
    """Centred integer frequencies -(m//2) .. m-m//2-1 (nufftfreqs1d, nufft_func.py:59-61)."""
    return df * np.arange(-(m // 2), m - (m // 2))


def _split(arr, ndim_spatial):
    """Return (array with trailing dims flattened to nt, trailing shape)."""
    trail = arr.shape[ndim_spatial:]
    nt = int(np.prod(trail)) if trail else 1
    return arr.reshape(arr.shape[:ndim_spatial] + (nt,)), trail


def _deapod(shape, tau, dim):
    """(pi/tau)^(dim/2) * exp(tau * |k|^2) on the ms x mt x mu image grid."""
    out = np.ones(shape, dtype=np.float64) * np.sqrt(np.pi / tau) ** dim
    for d, m in enumerate(shape):
        k = freqs(m)
        e = np.exp(tau * k ** 2)
        out = out * e.reshape((1,) * d + (m,) + (1,) * (dim - d - 1))
    return out


def _wrap_index(m, nf):
    return np.mod(freqs(m).astype(np.int64), nf)


def _pad(Fk_t, shape, nf):
    """Place an (nt, ms, mt, mu) image at frequency positions k mod nf (nufft_func.py:760-764)."""
    out = np.zeros((Fk_t.shape[0],) + tuple(nf), dtype=np.complex128)
    idx = np.ix_(np.arange(Fk_t.shape[0]), *[_wrap_index(m, n) for m, n in zip(shape, nf)])
    out[idx] = Fk_t
    return out


def _crop(F_t, shape, nf):
    """Inverse of _pad: the centred ms x mt x mu block (nufft_func.py:728-729)."""
    idx = np.ix_(np.arange(F_t.shape[0]), *[_wrap_index(m, n) for m, n in zip(shape, nf)])
    return F_t[idx]


def _fftn(a, axes, inverse, workers):
    if workers:
        import scipy.fft as sfft
        return (sfft.ifftn if inverse else sfft.fftn)(a, axes=axes, workers=workers)
    return (np.fft.ifftn if inverse else np.fft.fftn)(a, axes=axes)


# ---------------------------------------------------------------- tap loops

def spread(coords, c_t, tau, ns, nf):
    """Gridding (type-1 spread) of (nt, M) samples onto (nt,)+nf, FP64 (gridding.c)."""
    lib = _load()
    dim = len(nf)
    nt, M = c_t.shape
    c_t = np.ascontiguousarray(c_t, dtype=np.complex128)
    xs = [np.ascontiguousarray(v, dtype=np.float64) for v in coords]
    out = np.empty((nt,) + tuple(nf), dtype=np.complex128)
    i64 = ctypes.c_int64
    if dim == 1:
        lib.orc_spread1d(_ptr(xs[0]), _ptr(c_t), i64(M), nt, ctypes.c_double(tau), ns, i64(nf[0]), _ptr(out))
    elif dim == 2:
        lib.orc_spread2d(_ptr(xs[0]), _ptr(xs[1]), _ptr(c_t), i64(M), nt, ctypes.c_double(tau), ns,
                         i64(nf[0]), i64(nf[1]), _ptr(out))
    else:
        lib.orc_spread3d(_ptr(xs[0]), _ptr(xs[1]), _ptr(xs[2]), _ptr(c_t), i64(M), nt, ctypes.c_double(tau),
                         ns, i64(nf[0]), i64(nf[1]), i64(nf[2]), _ptr(out))
    return out


def interp(coords, grid_t, tau, ns):
    """Interpolation (type-2) of (nt,)+nf grids at M points, including the 1/N factor."""
    lib = _load()
    nf = grid_t.shape[1:]
    dim = len(nf)
    nt = grid_t.shape[0]
    M = len(coords[0])
    grid_t = np.ascontiguousarray(grid_t, dtype=np.complex128)
    xs = [np.ascontiguousarray(v, dtype=np.float64) for v in coords]
    out = np.empty((nt, M), dtype=np.complex128)
    i64 = ctypes.c_int64
    if dim == 1:
        lib.orc_interp1d(_ptr(xs[0]), _ptr(grid_t), i64(M), nt, ctypes.c_double(tau), ns, i64(nf[0]), _ptr(out))
    elif dim == 2:
        lib.orc_interp2d(_ptr(xs[0]), _ptr(xs[1]), _ptr(grid_t), i64(M), nt, ctypes.c_double(tau), ns,
                         i64(nf[0]), i64(nf[1]), _ptr(out))
    else:
        lib.orc_interp3d(_ptr(xs[0]), _ptr(xs[1]), _ptr(xs[2]), _ptr(grid_t), i64(M), nt, ctypes.c_double(tau),
                         ns, i64(nf[0]), i64(nf[1]), i64(nf[2]), _ptr(out))
    return out


def normal(coords, grid_t, tau, ns, dcf=None):
    """Per-sample interp -> (dcf/N) -> spread, the fused loop of build_grid_{1,2,3}d21."""
    lib = _load()
    nf = grid_t.shape[1:]
    dim = len(nf)
    nt = grid_t.shape[0]
    M = len(coords[0])
    grid_t = np.ascontiguousarray(grid_t, dtype=np.complex128)
    xs = [np.ascontiguousarray(v, dtype=np.float64) for v in coords]
    w = None if dcf is None else np.ascontiguousarray(dcf, dtype=np.float64).reshape(-1)
    out = np.empty_like(grid_t)
    i64 = ctypes.c_int64
    if dim == 1:
        lib.orc_normal1d(_ptr(xs[0]), _ptr(w), _ptr(grid_t), i64(M), nt, ctypes.c_double(tau), ns,
                         i64(nf[0]), _ptr(out))
    elif dim == 2:
        lib.orc_normal2d(_ptr(xs[0]), _ptr(xs[1]), _ptr(w), _ptr(grid_t), i64(M), nt, ctypes.c_double(tau), ns,
                         i64(nf[0]), i64(nf[1]), _ptr(out))
    else:
        lib.orc_normal3d(_ptr(xs[0]), _ptr(xs[1]), _ptr(xs[2]), _ptr(w), _ptr(grid_t), i64(M), nt,
                         ctypes.c_double(tau), ns, i64(nf[0]), i64(nf[1]), i64(nf[2]), _ptr(out))
    return out


# ---------------------------------------------------------------- drivers

def _params_for(dim, shape, eps):
    if dim == 3:
        return grid_params(3, *shape, eps=eps, max_nspread=6)
    return grid_params(dim, *shape, eps=eps)


def nufft_type1(coords, c, shape, df=1.0, eps=1e-15, iflag=1, workers=0):
    """(1/M) sum_j c_j exp(+/-i k.x_j) by Gaussian gridding: nufft{1,2,3}d1_gaussker."""
    dim = len(shape)
    ns, nf, tau = _params_for(dim, shape, eps)
    c2, trail = _split(np.asarray(c), 1)
    xs = [np.asarray(v, dtype=np.float64) * df for v in coords]
    F = spread(xs, c2.T, tau, ns, nf)
    axes = tuple(range(1, dim + 1))
    N = float(np.prod(nf))
    if iflag < 0:
        F = (1.0 / N) * _fftn(F, axes, False, workers)
    else:
        F = _fftn(F, axes, True, workers)
    F = _crop(F, shape, nf) * _deapod(shape, tau, dim)[None] * (1.0 / len(xs[0]))
    F = np.moveaxis(F, 0, -1)
    return F.reshape(tuple(shape) + trail)


def _type2_grid(Fk, shape, nf, tau, iflag, workers):
    dim = len(shape)
    F2, trail = _split(np.asarray(Fk), dim)
    Ft = np.moveaxis(F2, -1, 0) * _deapod(shape, tau, dim)[None]
    G = _pad(Ft, shape, nf)
    axes = tuple(range(1, dim + 1))
    if iflag < 0:
        G = float(np.prod(nf)) * _fftn(G, axes, True, workers)
    else:
        G = _fftn(G, axes, False, workers)
    return G, trail


def nufft_type2(coords, Fk, shape, df=1.0, eps=1e-15, iflag=1, workers=0):
    """sum_k F_k exp(-/+i k.x_j) by Gaussian gridding: nufft{1,2,3}d2_gaussker."""
    dim = len(shape)
    ns, nf, tau = _params_for(dim, shape, eps)
    G, trail = _type2_grid(Fk, shape, nf, tau, iflag, workers)
    xs = [np.asarray(v, dtype=np.float64) * df for v in coords]
    c = interp(xs, G, tau, ns)
    return c.T.reshape((len(xs[0]),) + trail)


def nufft_type21(coords, Fk, shape, dcf=None, df=1.0, eps=1e-15, iflag=1, workers=0):
    """(1/M) A^H D A F by the per-sample fused loop: nufft{1,2,3}d21_gaussker.

    The 1-D and 2-D reference drivers take no dcf (nufft_func.py:506, 780); pass
    dcf only for 3-D to follow the reference.  The 1-D driver's second FFT uses
    numpy's default last axis (nufft_func.py:538-540), which is axis 0 for the
    single-coil input it is written for; this restatement uses axis 0.
    """
    dim = len(shape)
    ns, nf, tau = _params_for(dim, shape, eps)
    G, trail = _type2_grid(Fk, shape, nf, tau, iflag, workers)
    xs = [np.asarray(v, dtype=np.float64) * df for v in coords]
    F = normal(xs, G, tau, ns, dcf)
    axes = tuple(range(1, dim + 1))
    N = float(np.prod(nf))
    if iflag < 0:
        F = (1.0 / N) * _fftn(F, axes, False, workers)
    else:
        F = _fftn(F, axes, True, workers)
    F = _crop(F, shape, nf) * _deapod(shape, tau, dim)[None] * (1.0 / len(xs[0]))
    F = np.moveaxis(F, 0, -1)
    return F.reshape(tuple(shape) + trail)


# ---------------------------------------------------------------- operator

class NUFFT3dOracle:
    """Restatement of pics/operators_class.py:302-364 (forward = type-2, backward =
    type-1 of dcf-weighted data, forward_backward = type-21 with dcf), eps 1e-5."""

    def __init__(self, im_shape, dcf=None):
        self.im_shape = tuple(im_shape)
        self.dcf = None if dcf is None else np.asarray(dcf).reshape(-1)
        self.kx = self.ky = self.kz = None

    def normalize_set_ktraj(self, ktraj):
        ktraj = np.pi * ktraj / ktraj.flatten().max()
        self.kx, self.ky, self.kz = (ktraj[i, :].flatten() for i in range(3))
        return self.kx, self.ky, self.kz

    def forward(self, im):
        return nufft_type2((self.kx, self.ky, self.kz), im, self.im_shape, eps=1e-5)

    def backward(self, kdata):
        w = self.dcf.reshape((-1,) + (1,) * (kdata.ndim - 1))
        return nufft_type1((self.kx, self.ky, self.kz), (kdata * w).squeeze(), self.im_shape, eps=1e-5)

    def forward_backward(self, im):
        return nufft_type21((self.kx, self.ky, self.kz), im, self.im_shape, dcf=self.dcf, eps=1e-5)


# ---------------------------------------------------------------- exact sums

def _kgrid(shape):
    return np.meshgrid(*[freqs(m) for m in shape], indexing="ij")


_CHUNK_ELEMS = 1 << 23  # complex128 phase entries per chunk (128 MiB)


def nudft_type1(coords, c, shape, df=1.0, iflag=1, pixels=None):
    """(1/M) sum_j c_j exp(s i k.x_j), s = sign(iflag) (nudft{1,2,3}d1).
    pixels: optional flat indices into the image; then returns (len(pixels), *trail).
    Memory is bounded by chunking over samples."""
    s = -1.0 if iflag < 0 else 1.0
    ks = [k.reshape(-1) for k in _kgrid(shape)]
    if pixels is not None:
        ks = [k[np.asarray(pixels)] for k in ks]
    xs = [np.asarray(v, dtype=np.float64).reshape(-1) * df for v in coords]
    c2, trail = _split(np.asarray(c), 1)
    M, K = len(xs[0]), len(ks[0])
    out = np.zeros((K, c2.shape[1]), dtype=np.complex128)
    step = max(1, _CHUNK_ELEMS // max(K, 1))
    for a in range(0, M, step):
        phase = sum(k[:, None] * x[None, a:a + step] for k, x in zip(ks, xs))   # (K, m)
        out += np.exp(s * 1j * phase) @ c2[a:a + step]
    out /= M
    return out.reshape((K,) + trail) if pixels is not None else out.reshape(tuple(shape) + trail)


def nudft_type2(coords, Fk, shape, df=1.0, iflag=1):
    """sum_k F_k exp(-s i k.x_j): the exact operator that type-2 approximates."""
    s = -1.0 if iflag < 0 else 1.0
    dim = len(shape)
    ks = [k.reshape(-1) for k in _kgrid(shape)]
    xs = [np.asarray(v, dtype=np.float64).reshape(-1) * df for v in coords]
    F2, trail = _split(np.asarray(Fk), dim)
    F2 = F2.reshape(-1, F2.shape[-1])
    M, K = len(xs[0]), len(ks[0])
    out = np.empty((M, F2.shape[1]), dtype=np.complex128)
    step = max(1, _CHUNK_ELEMS // max(K, 1))
    for a in range(0, M, step):
        phase = sum(x[a:a + step, None] * k[None, :] for k, x in zip(ks, xs))   # (m, K)
        out[a:a + step] = np.exp(-s * 1j * phase) @ F2
    return out.reshape((M,) + trail)


def nudft_type2_coord_grad(coords, Fk, shape, grad_c, df=1.0, iflag=1):
    """d/dx_{j,d} of Re<grad_c, A(x) F>, i.e. Re(conj(grad_c_j) . dc_j/dx_{j,d}) summed over
    coils, for the exact type-2 sum.  Returns (M, dim) float64."""
    s = -1.0 if iflag < 0 else 1.0
    dim = len(shape)
    ks = [k.reshape(-1) for k in _kgrid(shape)]
    xs = [np.asarray(v, dtype=np.float64).reshape(-1) * df for v in coords]
    F2, _ = _split(np.asarray(Fk), dim)
    F2 = F2.reshape(-1, F2.shape[-1])
    M, K = len(xs[0]), len(ks[0])
    g2 = np.asarray(grad_c).reshape(M, -1)
    out = np.empty((M, dim))
    step = max(1, _CHUNK_ELEMS // max(K, 1))
    for a in range(0, M, step):
        E = np.exp(-s * 1j * sum(x[a:a + step, None] * k[None, :] for k, x in zip(ks, xs)))
        for d in range(dim):
            dc = (E * (-s * 1j * ks[d][None, :])) @ F2                         # (m, nt)
            out[a:a + step, d] = np.real(np.conj(g2[a:a + step]) * dc).sum(axis=1) * df
    return out


# ---------------------------------------------------------------- exact sums, separable forms
# The same exact sums as nudft_type1 / nudft_type2, arranged so that full-size checks
# (millions of samples, 128^3 images) finish in seconds: the phase exp(s i k.x) is the
# product of one factor per axis, so the sums contract one axis at a time as matrix
# products instead of forming the (pixels x samples) phase matrix.

def _axis_phase(x, m, s):
    """exp(s i k x) for the centred frequencies k of one axis: (len(x), m) complex128."""
    return np.exp(s * 1j * np.multiply.outer(np.asarray(x, dtype=np.float64), freqs(m)))


def nudft_type2_at(coords, Fk, shape, samples, df=1.0, iflag=1, chunk=64):
    """sum_k F_k exp(-s i k.x_j) for the listed sample indices only (exact, FP64).
    Fk: (*shape, *trail).  Returns (len(samples), *trail)."""
    s = -1.0 if iflag < 0 else 1.0
    dim = len(shape)
    F2, trail = _split(np.asarray(Fk, dtype=np.complex128), dim)
    nt = F2.shape[-1]
    idx = np.asarray(samples, dtype=np.int64)
    xs = [np.asarray(v, dtype=np.float64)[idx] * df for v in coords]
    out = np.empty((len(idx), nt), dtype=np.complex128)
    for a in range(0, len(idx), chunk):
        b = min(a + chunk, len(idx))
        # last axis: (n, m_last) @ (m_last, rest) with the axis moved to the front
        E = _axis_phase(xs[dim - 1][a:b], shape[dim - 1], -s)
        T = np.moveaxis(F2, dim - 1, 0).reshape(shape[dim - 1], -1)
        T = (E @ T).reshape((b - a,) + tuple(shape[:dim - 1]) + (nt,))
        for d in range(dim - 2, -1, -1):
            E = _axis_phase(xs[d][a:b], shape[d], -s)              # (n, m_d)
            T = np.einsum("n...kc,nk->n...c", T, E)                # contract axis d (the last spatial one left)
        out[a:b] = T.reshape(b - a, nt)
    return out.reshape((len(idx),) + trail)


def nudft_type1_box(coords, c, shape, pix_axes, df=1.0, iflag=1, chunk=1 << 16):
    """(1/M) sum_j c_j exp(s i k.x_j) at the pixels of a box: the outer product of the
    per-axis index lists pix_axes[d] (indices into the image axis d).  Exact, FP64.
    c: (M, *trail).  Returns (len(pix_axes[0]), ..., *trail)."""
    s = -1.0 if iflag < 0 else 1.0
    dim = len(shape)
    xs = [np.asarray(v, dtype=np.float64).reshape(-1) * df for v in coords]
    c2, trail = _split(np.asarray(c, dtype=np.complex128), 1)
    M, nt = c2.shape
    ks = [freqs(m)[np.asarray(p, dtype=np.int64)] for m, p in zip(shape, pix_axes)]
    sizes = [len(k) for k in ks]
    # split the axes into two groups: left = the first half, right = the rest and the coils;
    # per chunk  out[left, right] += L^T R  with  L[j] = prod of left phases (outer product)
    # and  R[j] = prod of right phases x c_j, so the (pixels x samples) products run in BLAS
    h = (dim + 1) // 2
    out = np.zeros((int(np.prod(sizes[:h])), int(np.prod(sizes[h:])) * nt), dtype=np.complex128)
    for a in range(0, M, chunk):
        b = min(a + chunk, M)
        n = b - a
        L = np.ones((n, 1), dtype=np.complex128)
        for d in range(h):
            Ed = np.exp(s * 1j * np.multiply.outer(xs[d][a:b], ks[d]))
            L = (L[:, :, None] * Ed[:, None, :]).reshape(n, -1)
        R = np.ones((n, 1), dtype=np.complex128)
        for d in range(h, dim):
            Ed = np.exp(s * 1j * np.multiply.outer(xs[d][a:b], ks[d]))
            R = (R[:, :, None] * Ed[:, None, :]).reshape(n, -1)
        R = (R[:, :, None] * c2[a:b][:, None, :]).reshape(n, -1)
        out += L.T @ R
    out /= M
    return out.reshape(tuple(sizes) + trail)
