"""Generate the golden NUFFT vectors in ``tests/golden/*.npz`` from mripy's own CPU code.

This script is test infrastructure.  It runs the reference implementation
(peng-cao/mripy ``fft/nufft_func.py`` and ``pics/operators_class.py``) in a
container that has the reference checked out, and writes small input/output
fixtures that the oracle and the GPU parity tests compare against.  The GPU
box never runs it: the fixtures travel, the reference does not.

mripy imports packages that are not installed here (numba, matplotlib,
pyFFTW, PyWavelets).  None of them carries NUFFT arithmetic, so tiny stand-ins
are registered before the import:

* ``numba``: ``jit``/``njit`` return the function unchanged, ``prange`` is
  ``range`` and ``numba.cuda.is_available()`` is False.  The decorated loops
  then run as plain Python with float64/complex128 numpy scalars, which is the
  arithmetic numba would compile.
* ``pyfftw``: ``FFTW(a, b, axes, direction)`` calls ``numpy.fft.fftn`` /
  ``ifftn``.  pyFFTW 0.10.4 (the version pinned in mripy's
  ``env_requirements.txt``) normalises inverse transforms in ``FFTW.__call__``
  (``normalise_idft=True``), like ``numpy.fft.ifftn``.
* ``matplotlib`` and ``pywt``: no-op modules (plotting and wavelets only).

Usage:  python tests/golden/make_golden.py /path/to/mripy
        (or set MRIPY_REFERENCE to the checkout's root and omit the argument)
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _install_stubs():
    numba = types.ModuleType("numba")

    def _identity_decorator(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    numba.jit = _identity_decorator
    numba.njit = _identity_decorator
    numba.prange = range
    cuda = types.ModuleType("numba.cuda")
    cuda.is_available = lambda: False
    cuda.jit = _identity_decorator
    numba.cuda = cuda
    sys.modules["numba"] = numba
    sys.modules["numba.cuda"] = cuda

    mpl = types.ModuleType("matplotlib")
    mpl.use = lambda *a, **k: None
    plt = types.ModuleType("matplotlib.pyplot")
    cm = types.ModuleType("matplotlib.cm")
    mpl.pyplot = plt
    mpl.cm = cm
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt
    sys.modules["matplotlib.cm"] = cm

    pyfftw = types.ModuleType("pyfftw")

    class FFTW:
        def __init__(self, a, b, axes=(0,), direction="FFTW_FORWARD", threads=1):
            self.a, self.axes, self.direction = a, tuple(axes), direction

        def __call__(self):
            if self.direction == "FFTW_BACKWARD":
                return np.fft.ifftn(self.a, axes=self.axes)
            return np.fft.fftn(self.a, axes=self.axes)

    pyfftw.FFTW = FFTW
    pyfftw.empty_aligned = lambda shape, dtype=None: np.empty(shape, dtype=dtype)
    interfaces = types.ModuleType("pyfftw.interfaces")
    cache = types.ModuleType("pyfftw.interfaces.cache")
    cache.enable = lambda: None
    interfaces.cache = cache
    pyfftw.interfaces = interfaces
    sys.modules["pyfftw"] = pyfftw
    sys.modules["pyfftw.interfaces"] = interfaces
    sys.modules["pyfftw.interfaces.cache"] = cache

    sys.modules["pywt"] = types.ModuleType("pywt")


def reference_root():
    """The mripy checkout to run: the first command-line argument, else $MRIPY_REFERENCE."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MRIPY_REFERENCE")
    if not root or not os.path.isdir(os.path.join(root, "fft")):
        sys.exit("usage: %s /path/to/mripy  (or set MRIPY_REFERENCE)" % os.path.basename(sys.argv[0]))
    return root


def load_reference(ref_root):
    _install_stubs()
    sys.path.insert(0, os.path.join(ref_root, "fft"))
    sys.path.insert(0, ref_root)
    import warnings
    warnings.simplefilter("ignore", SyntaxWarning)
    import fft.nufft_func as nft  # noqa: E402
    import pics.operators_class as opc  # noqa: E402
    return nft, opc


def _rand_complex(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _silence(fn, *a, **k):
    # the reference prints timings; keep the generator output readable
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def make_1d(nft):
    out = {}
    rng = np.random.RandomState(0)
    M, ms = 300, 20
    x = 100 * rng.rand(M)                       # outside [-pi, pi): exercises the mod-2pi wrap
    c = 1j * np.sin(x) + 1j * np.sin(10 * x)
    Fk = _rand_complex(rng, (ms,))
    out["x"], out["c"], out["Fk"] = x, c, Fk
    out["ms"] = np.int64(ms)
    for eps, tag in ((5e-6, "e5em6"), (1e-3, "e1em3")):
        for df in (1.0, 2.0):
            for iflag in (1, -1):
                key = "%s_df%d_if%+d" % (tag, int(df), iflag)
                out["t1_" + key] = nft.nufft1d1_gaussker(x, c, ms, df=df, eps=eps, iflag=iflag)
                out["t2_" + key] = nft.nufft1d2_gaussker(x, Fk, ms, df=df, eps=eps, iflag=iflag)
                out["t21_" + key] = nft.nufft1d21_gaussker(x, Fk, ms, df=df, eps=eps, iflag=iflag)
    out["nudft1d1"] = nft.nudft1d1(x, c, ms)
    return out


def make_2d(nft):
    out = {}
    # case a: the reference's own test recipe (nufft_test_func.compare_nufft2d1)
    rng = np.random.RandomState(0)
    M, ms, mt = 400, 16, 16
    x = 100 * rng.rand(M)
    y = 100 * rng.rand(M)
    c = np.sin(2 * x) + 1j * np.cos(2 * y)
    Fk = _rand_complex(rng, (ms, mt))
    out.update(a_x=x, a_y=y, a_c=c, a_Fk=Fk, a_ms=np.int64(ms), a_mt=np.int64(mt))
    for eps, tag in ((5e-6, "e5em6"), (1e-5, "e1em5")):
        for df in (1.0, 2.0):
            for iflag in (1, -1):
                key = "a_%s_df%d_if%+d" % (tag, int(df), iflag)
                out["t1_" + key] = nft.nufft2d1_gaussker(x, y, c, ms, mt, df=df, eps=eps, iflag=iflag)
                out["t2_" + key] = nft.nufft2d2_gaussker(x, y, Fk, ms, mt, df=df, eps=eps, iflag=iflag)
                out["t21_" + key] = nft.nufft2d21_gaussker(x, y, Fk, ms, mt, df=df, eps=eps, iflag=iflag)
    out["a_nudft2d1"] = nft.nudft2d1(x, y, c, ms, mt)
    out["a_nudft2d1_if-1"] = nft.nudft2d1(x, y, c, ms, mt, iflag=-1)

    # case b: non-square, odd sizes, coil-last trailing dimension, points in [-pi, pi)
    rng = np.random.RandomState(1)
    M, ms, mt, nc = 300, 15, 12, 3
    x = np.pi * (2 * rng.rand(M) - 1)
    y = np.pi * (2 * rng.rand(M) - 1)
    c = _rand_complex(rng, (M, nc))
    Fk = _rand_complex(rng, (ms, mt, nc))
    out.update(b_x=x, b_y=y, b_c=c, b_Fk=Fk, b_ms=np.int64(ms), b_mt=np.int64(mt))
    for eps, tag in ((1e-5, "e1em5"), (1e-3, "e1em3")):
        key = "b_%s" % tag
        out["t1_" + key] = nft.nufft2d1_gaussker(x, y, c, ms, mt, eps=eps)
        # nufft2d2_gaussker allocates its output as np.zeros(x.shape) (nufft_func.py:612),
        # so the reference takes one coil per call: stack the per-coil results
        out["t2_" + key] = np.stack([nft.nufft2d2_gaussker(x, y, Fk[..., k], ms, mt, eps=eps)
                                     for k in range(nc)], axis=-1)
        out["t21_" + key] = nft.nufft2d21_gaussker(x, y, Fk, ms, mt, eps=eps)
    return out


def make_3d(nft, opc):
    out = {}
    rng = np.random.RandomState(0)
    M, ms, mt, mu = 150, 8, 8, 6
    x = 100 * rng.rand(M)
    y = 100 * rng.rand(M)
    z = 100 * rng.rand(M)
    c = np.sin(2 * x) + 1j * np.cos(2 * y)
    Fk = _rand_complex(rng, (ms, mt, mu))
    dcf = 0.5 + rng.rand(M)
    out.update(a_x=x, a_y=y, a_z=z, a_c=c, a_Fk=Fk, a_dcf=dcf,
               a_ms=np.int64(ms), a_mt=np.int64(mt), a_mu=np.int64(mu))
    for eps, tag in ((5e-6, "e5em6"), (1e-5, "e1em5")):
        for iflag in (1, -1):
            key = "a_%s_if%+d" % (tag, iflag)
            out["t1_" + key] = _silence(nft.nufft3d1_gaussker, x, y, z, c, ms, mt, mu, eps=eps, iflag=iflag)
            out["t2_" + key] = _silence(nft.nufft3d2_gaussker, x, y, z, Fk, ms, mt, mu, eps=eps, iflag=iflag)
            # build_grid_3d21_wrap's single-coil branch drops build_grid_3d21's return value
            # (nufft_func.py:1115-1116) and hands back the un-gridded input; the multi-coil
            # branch (and the CUDA twin, nufft_func_cuda.py:1358-1359) is correct, so the
            # golden goes through it with a trailing singleton coil axis.
            out["t21_" + key] = _silence(nft.nufft3d21_gaussker, x, y, z, Fk[..., None], ms, mt, mu,
                                         dcf=dcf, eps=eps, iflag=iflag)[..., 0]
    # eps below the 3-D clamp: nspread is capped at 6 by max_nspread
    out["t1_a_e1em12_if+1"] = _silence(nft.nufft3d1_gaussker, x, y, z, c, ms, mt, mu, eps=1e-12)
    out["a_nudft3d1"] = nft.nudft3d1(x, y, z, c, ms, mt, mu)

    # case b: multi-coil through the NUFFT3d operator class (eps 1e-5, dcf weighting)
    rng = np.random.RandomState(2)
    M, ms, mt, mu, nc = 120, 8, 6, 6, 2
    ktraj = rng.rand(3, M) - 0.5
    dcf = 0.5 + rng.rand(M)
    im = _rand_complex(rng, (ms, mt, mu, nc))
    kd = _rand_complex(rng, (M, nc))
    op = opc.NUFFT3d((ms, mt, mu), dcf)
    kx, ky, kz = op.normalize_set_ktraj(ktraj.copy())
    out.update(b_ktraj=ktraj, b_dcf=dcf, b_im=im, b_kdata=kd, b_kx=kx, b_ky=ky, b_kz=kz,
               b_shape=np.array([ms, mt, mu], np.int64))
    out["b_forward"] = _silence(op.forward, im)
    out["b_backward"] = _silence(op.backward, kd)
    out["b_forward_backward"] = _silence(op.forward_backward, im)
    return out


def main():
    ref_root = reference_root()
    nft, opc = load_reference(ref_root)
    for name, data in (("golden_1d.npz", make_1d(nft)),
                       ("golden_2d.npz", make_2d(nft)),
                       ("golden_3d.npz", make_3d(nft, opc))):
        path = os.path.join(HERE, name)
        np.savez_compressed(path, **data)
        print("wrote", path, "keys:", len(data), "bytes:", os.path.getsize(path))


if __name__ == "__main__":
    main()
