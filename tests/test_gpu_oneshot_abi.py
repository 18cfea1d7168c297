"""The one-shot C entry points gbn_nufft{2,3}d{1,2,21}_gaussker, bound with plain ctypes
exactly as a mripy maintainer would bind them (the module shown in INTEGRATION.md):
host float64 coordinates, host complex64 data with trailing coils, host output, no torch.
Each call uploads the coordinates, sorts them, runs the transform on its own stream,
converts the 3-D dcf from float64 and writes the coil-last result back.

Reference signatures: fft/nufft_func_cuda.py:581, 609, 639 (2-D), 1463, 1512, 1562 (3-D);
the expected values are mripy's own outputs (tests/golden, made by make_golden.py from
fft/nufft_func.py and pics/operators_class.py).

Tolerance: TOL_REF = 2e-5 relative L2 (complex64 data and FP32 stencils against mripy's
complex128 result at the same eps).
"""
import ctypes
import os

import numpy as np
import pytest

from mripy_gb300 import _native

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden")
TOL_REF = 2e-5

_c = ctypes
_ARGS_2D = [_c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_int64, _c.c_int32, _c.c_int32, _c.c_int32, _c.c_double,
            _c.c_double, _c.c_int32, _c.c_void_p]
_ARGS_3D = [_c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_int64, _c.c_int32, _c.c_int32, _c.c_int32,
            _c.c_int32, _c.c_double, _c.c_double, _c.c_int32, _c.c_void_p]
_ARGS_3D21 = [_c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_int64, _c.c_int32, _c.c_int32, _c.c_int32,
              _c.c_int32, _c.c_void_p, _c.c_double, _c.c_double, _c.c_int32, _c.c_void_p]


@pytest.fixture(scope="module")
def lib():
    L = ctypes.CDLL(_native.LIB_PATH)          # a fresh binding: nothing from the package's wrapper
    for name in ("gbn_nufft2d1_gaussker", "gbn_nufft2d2_gaussker", "gbn_nufft2d21_gaussker"):
        getattr(L, name).argtypes = _ARGS_2D
        getattr(L, name).restype = _c.c_int32
    for name in ("gbn_nufft3d1_gaussker", "gbn_nufft3d2_gaussker"):
        getattr(L, name).argtypes = _ARGS_3D
        getattr(L, name).restype = _c.c_int32
    L.gbn_nufft3d21_gaussker.argtypes = _ARGS_3D21
    L.gbn_nufft3d21_gaussker.restype = _c.c_int32
    return L


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _f64(a):
    return np.ascontiguousarray(a, np.float64)


def _c64(a):
    return np.ascontiguousarray(a, np.complex64)


def _ntrail(a, lead):
    return int(np.prod(a.shape[lead:])) if a.ndim > lead else 1


# --- the binding module a maintainer would add to mripy (fft/nufft_gb300.py), verbatim in spirit
def nufft2d1(L, x, y, c, ms, mt, df=1.0, eps=1e-15, iflag=1):
    x, y, c = _f64(x), _f64(y), _c64(c)
    out = np.empty((ms, mt) + c.shape[1:], np.complex64)
    st = L.gbn_nufft2d1_gaussker(x.ctypes.data, y.ctypes.data, c.ctypes.data, len(x), _ntrail(c, 1), ms, mt, df,
                                 eps, iflag, out.ctypes.data)
    assert st == 0, st
    return out.astype(np.complex128)


def nufft2d2(L, x, y, Fk, ms, mt, df=1.0, eps=1e-15, iflag=1):
    x, y, Fk = _f64(x), _f64(y), _c64(Fk)
    out = np.empty((len(x),) + Fk.shape[2:], np.complex64)
    st = L.gbn_nufft2d2_gaussker(x.ctypes.data, y.ctypes.data, Fk.ctypes.data, len(x), _ntrail(Fk, 2), ms, mt, df,
                                 eps, iflag, out.ctypes.data)
    assert st == 0, st
    return out.astype(np.complex128)


def nufft2d21(L, x, y, Fk, ms, mt, df=1.0, eps=1e-15, iflag=1):
    x, y, Fk = _f64(x), _f64(y), _c64(Fk)
    out = np.empty(Fk.shape, np.complex64)
    st = L.gbn_nufft2d21_gaussker(x.ctypes.data, y.ctypes.data, Fk.ctypes.data, len(x), _ntrail(Fk, 2), ms, mt, df,
                                  eps, iflag, out.ctypes.data)
    assert st == 0, st
    return out.astype(np.complex128)


def nufft3d1(L, x, y, z, c, ms, mt, mu, df=1.0, eps=1e-15, iflag=1):
    x, y, z, c = _f64(x), _f64(y), _f64(z), _c64(c)
    out = np.empty((ms, mt, mu) + c.shape[1:], np.complex64)
    st = L.gbn_nufft3d1_gaussker(x.ctypes.data, y.ctypes.data, z.ctypes.data, c.ctypes.data, len(x), _ntrail(c, 1),
                                 ms, mt, mu, df, eps, iflag, out.ctypes.data)
    assert st == 0, st
    return out.astype(np.complex128)


def nufft3d2(L, x, y, z, Fk, ms, mt, mu, df=1.0, eps=1e-15, iflag=1):
    x, y, z, Fk = _f64(x), _f64(y), _f64(z), _c64(Fk)
    out = np.empty((len(x),) + Fk.shape[3:], np.complex64)
    st = L.gbn_nufft3d2_gaussker(x.ctypes.data, y.ctypes.data, z.ctypes.data, Fk.ctypes.data, len(x),
                                 _ntrail(Fk, 3), ms, mt, mu, df, eps, iflag, out.ctypes.data)
    assert st == 0, st
    return out.astype(np.complex128)


def nufft3d21(L, x, y, z, Fk, ms, mt, mu, dcf=None, df=1.0, eps=1e-15, iflag=1):
    x, y, z, Fk = _f64(x), _f64(y), _f64(z), _c64(Fk)
    w = None if dcf is None else _f64(dcf)
    out = np.empty(Fk.shape, np.complex64)
    st = L.gbn_nufft3d21_gaussker(x.ctypes.data, y.ctypes.data, z.ctypes.data, Fk.ctypes.data, len(x),
                                  _ntrail(Fk, 3), ms, mt, mu, None if w is None else w.ctypes.data, df, eps, iflag,
                                  out.ctypes.data)
    assert st == 0, st
    return out.astype(np.complex128)


# ------------------------------------------------------------------ 2-D
@pytest.mark.parametrize("eps,tag", [(5e-6, "e5em6"), (1e-5, "e1em5")])
@pytest.mark.parametrize("df", [1.0, 2.0])
@pytest.mark.parametrize("iflag", [1, -1])
def test_oneshot_2d_single_coil(lib, eps, tag, df, iflag):
    g = np.load(os.path.join(G, "golden_2d.npz"))
    x, y, c, Fk = g["a_x"], g["a_y"], g["a_c"], g["a_Fk"]
    ms, mt = int(g["a_ms"]), int(g["a_mt"])
    key = "a_%s_df%d_if%+d" % (tag, int(df), iflag)
    assert rel(nufft2d1(lib, x, y, c, ms, mt, df, eps, iflag), g["t1_" + key]) < TOL_REF
    assert rel(nufft2d2(lib, x, y, Fk, ms, mt, df, eps, iflag), g["t2_" + key]) < TOL_REF
    assert rel(nufft2d21(lib, x, y, Fk, ms, mt, df, eps, iflag), g["t21_" + key]) < TOL_REF


@pytest.mark.parametrize("eps,tag", [(1e-5, "e1em5"), (1e-3, "e1em3")])
def test_oneshot_2d_trailing_coils(lib, eps, tag):
    g = np.load(os.path.join(G, "golden_2d.npz"))
    x, y, c, Fk = g["b_x"], g["b_y"], g["b_c"], g["b_Fk"]      # 3 coils, last axis
    ms, mt = int(g["b_ms"]), int(g["b_mt"])
    assert rel(nufft2d1(lib, x, y, c, ms, mt, eps=eps), g["t1_b_" + tag]) < TOL_REF
    assert rel(nufft2d2(lib, x, y, Fk, ms, mt, eps=eps), g["t2_b_" + tag]) < TOL_REF
    assert rel(nufft2d21(lib, x, y, Fk, ms, mt, eps=eps), g["t21_b_" + tag]) < TOL_REF


# ------------------------------------------------------------------ 3-D
@pytest.mark.parametrize("eps,tag", [(5e-6, "e5em6"), (1e-5, "e1em5")])
@pytest.mark.parametrize("iflag", [1, -1])
def test_oneshot_3d_with_dcf(lib, eps, tag, iflag):
    g = np.load(os.path.join(G, "golden_3d.npz"))
    x, y, z, c, Fk, dcf = (g[k] for k in ("a_x", "a_y", "a_z", "a_c", "a_Fk", "a_dcf"))
    ms, mt, mu = int(g["a_ms"]), int(g["a_mt"]), int(g["a_mu"])
    key = "a_%s_if%+d" % (tag, iflag)
    assert rel(nufft3d1(lib, x, y, z, c, ms, mt, mu, eps=eps, iflag=iflag), g["t1_" + key]) < TOL_REF
    assert rel(nufft3d2(lib, x, y, z, Fk, ms, mt, mu, eps=eps, iflag=iflag), g["t2_" + key]) < TOL_REF
    assert rel(nufft3d21(lib, x, y, z, Fk, ms, mt, mu, dcf=dcf, eps=eps, iflag=iflag), g["t21_" + key]) < TOL_REF


def test_oneshot_3d_operator_case_trailing_coils(lib):
    """The NUFFT3d operator's three calls (pics/operators_class.py:330-364: forward = type-2,
    backward = type-1 of dcf-weighted data, forward_backward = type-21 with dcf) through the
    one-shot entry points, 2 trailing coils, eps 1e-5."""
    g = np.load(os.path.join(G, "golden_3d.npz"))
    kx, ky, kz, dcf = g["b_kx"], g["b_ky"], g["b_kz"], g["b_dcf"]
    shp = tuple(int(v) for v in g["b_shape"])
    assert rel(nufft3d2(lib, kx, ky, kz, g["b_im"], *shp, eps=1e-5), g["b_forward"]) < TOL_REF
    assert rel(nufft3d1(lib, kx, ky, kz, g["b_kdata"] * dcf[:, None], *shp, eps=1e-5), g["b_backward"]) < TOL_REF
    assert rel(nufft3d21(lib, kx, ky, kz, g["b_im"], *shp, dcf=dcf, eps=1e-5), g["b_forward_backward"]) < TOL_REF


def test_oneshot_rejects_bad_arguments(lib):
    """Status codes, no exceptions, for arguments the reference would fail on."""
    x = np.zeros(4)
    c = np.zeros(4, np.complex64)
    out = np.zeros((8, 8), np.complex64)
    assert lib.gbn_nufft2d1_gaussker(x.ctypes.data, x.ctypes.data, c.ctypes.data, 4, 1, 8, 8, 1.0, 0.5, 1,
                                     out.ctypes.data) != 0          # eps outside (1e-33, 1e-1)
    assert lib.gbn_nufft2d1_gaussker(None, x.ctypes.data, c.ctypes.data, 4, 1, 8, 8, 1.0, 1e-5, 1,
                                     out.ctypes.data) != 0          # missing coordinates
