"""Generate ``tests/golden/golden_solvers.npz`` and ``golden_espirit.npz`` from mripy's own
solver and ESPIRiT code.

This script is test infrastructure, run where a mripy checkout is available; the
fixtures travel, the reference does not.  It runs the reference functions themselves:

* pics/CS_MRI_solvers_func.py   IST_32, FIST_32 (:75-86, 207-224), IST_3, FIST_3, IST_2,
                                FIST_2, ADMM_l2Afxnb_l1x, ADMM_l2Afxnb_l1Tfx, ADMM_l2Afxnb_l1x_2
* pics/proximal_func.py         prox_l1_soft_thresh, prox_l1_soft_thresh2, prox_l2_Afxnb_GD,
                                prox_l2_Afxnb_CGD (:282-311)
* pics/opt_alg.py               BacktrackingLineSearch (:8-33)
* espirit/espirit_func.py       espirit_2d (:25-119), espirit_3d (:122-219)

on small problems: a dense complex operator A (96 x 64) acting on an 8 x 8 image, with
sparsifying transforms T = a random unitary matrix or the level-2 Haar transform, and
synthetic multi-coil k-space for ESPIRiT.

Those files are Python 2.  They are loaded through an import hook that makes the few
Python-2 constructs they use run under Python 3 with Python 2's meaning, without touching
the arithmetic: ``print x`` statements become ``print(x)``; ``/`` between two integers
(Python ints or numpy integer scalars or arrays) floors, as Python 2 did; ``map`` returns a
list.  numpy 2 has no ``np.int``; it is set to ``int`` (its Python 2 meaning), and
``scipy.signal.hamming`` (the symmetric Hamming window) is found at its later home
``scipy.signal.windows.hamming``.  The
reference's ``espirit_2d`` reads an undefined name ``nsing_th`` (:48); it is given the
value of the function's ``nsigv_th`` default (0.2), which ``espirit_3d`` uses in the same
place.  PyWavelets is not installed: the Haar transform handed to the solvers as T is the
oracle's restatement (oracle/solver_oracle.py, pinned by known answers of the published
transform); the unitary-matrix cases pin the solver loops independently of it.
matplotlib, numba and pyFFTW are stubbed as in make_golden.py (pyFFTW by numpy.fft with
its normalised inverse).

Usage:  python tests/golden/make_golden_solvers.py /path/to/mripy
        (or set MRIPY_REFERENCE to the checkout's root and omit the argument)
"""
import ast
import contextlib
import importlib.abc
import importlib.machinery
import importlib.util
import io
import os
import re
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)

import make_golden as MG  # noqa: E402


# ------------------------------------------------------------------ Python 2 semantics
def _py2_div(a, b):
    def is_int(v):
        if isinstance(v, bool):
            return False
        if isinstance(v, (int, np.integer)):
            return True
        return isinstance(v, np.ndarray) and np.issubdtype(v.dtype, np.integer)
    return a // b if is_int(a) and is_int(b) else a / b


def _py2_map(*a):
    return list(map(*a))


class _Py2Transformer(ast.NodeTransformer):
    def visit_BinOp(self, node):
        self.generic_visit(node)
        if isinstance(node.op, ast.Div):
            return ast.copy_location(ast.Call(func=ast.Name("__py2_div__", ast.Load()), args=[node.left, node.right],
                                              keywords=[]), node)
        return node

    def visit_AugAssign(self, node):
        self.generic_visit(node)
        if isinstance(node.op, ast.Div):
            tgt = node.target
            load = ast.Name(tgt.id, ast.Load()) if isinstance(tgt, ast.Name) else None
            if load is not None:
                return ast.copy_location(ast.Assign(targets=[tgt], value=ast.Call(
                    func=ast.Name("__py2_div__", ast.Load()), args=[load, node.value], keywords=[])), node)
        return node

    def visit_Call(self, node):
        self.generic_visit(node)
        if isinstance(node.func, ast.Name) and node.func.id == "map":
            node.func = ast.Name("__py2_map__", ast.Load())
        return node


_PRINT = re.compile(r"^(\s*)print\s+(?![\(=])(.*?)\s*$", re.M)


def py2_source_to_code(source, path):
    src = _PRINT.sub(r"\1print(\2)", source)
    tree = _Py2Transformer().visit(ast.parse(src, filename=path))
    ast.fix_missing_locations(tree)
    return compile(tree, path, "exec", dont_inherit=True)


class _Py2Loader(importlib.machinery.SourceFileLoader):
    def get_code(self, fullname):
        path = self.get_filename(fullname)
        return py2_source_to_code(self.get_data(path).decode("utf-8", "replace"), path)

    def exec_module(self, module):
        module.__dict__["__py2_div__"] = _py2_div
        module.__dict__["__py2_map__"] = _py2_map
        super().exec_module(module)


class _Py2Finder(importlib.abc.MetaPathFinder):
    """Loads every module that resolves to a file under the reference root with _Py2Loader."""

    def __init__(self, root):
        self.root = os.path.realpath(root)

    def find_spec(self, fullname, path=None, target=None):
        spec = importlib.machinery.PathFinder.find_spec(fullname, path)
        if spec is None or not spec.origin or not spec.origin.endswith(".py"):
            return None
        if not os.path.realpath(spec.origin).startswith(self.root + os.sep):
            return None
        spec.loader = _Py2Loader(fullname, spec.origin)
        return spec


class _Inert:
    """Stands in for any matplotlib object: every attribute, call and unpacking gives
    another inert object, so plotting calls (fig, ax = plt.subplots(); ax.imshow(...))
    do nothing."""

    def __getattr__(self, name):
        return _Inert()

    def __call__(self, *a, **k):
        return _Inert()

    def __iter__(self):
        return iter((_Inert(), _Inert()))


def _quiet_matplotlib():
    """No-op matplotlib whose every attribute is an inert object."""
    for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.cm", "matplotlib.colors"):
        m = types.ModuleType(name)
        m.__getattr__ = lambda attr: _Inert()
        sys.modules[name] = m
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    sys.modules["matplotlib"].cm = sys.modules["matplotlib.cm"]


def load(ref_root):
    MG._install_stubs()
    _quiet_matplotlib()
    if not hasattr(np, "int"):
        np.int = int
    import scipy.signal
    if not hasattr(scipy.signal, "hamming"):
        scipy.signal.hamming = scipy.signal.windows.hamming   # moved there by later scipy releases
    sys.dont_write_bytecode = True
    sys.meta_path.insert(0, _Py2Finder(ref_root))
    for sub in ("", "pics", "fft", "utilities", "espirit", "signal_processing", "dwt"):
        sys.path.insert(0, os.path.join(ref_root, sub) if sub else ref_root)
    import pics.CS_MRI_solvers_func as solvers  # noqa: E402
    import pics.proximal_func as pf  # noqa: E402
    import pics.opt_alg as alg  # noqa: E402
    import espirit.espirit_func as esp  # noqa: E402
    if not hasattr(esp, "nsing_th"):
        esp.nsing_th = 0.2        # espirit_2d's undefined name: the nsigv_th default, as espirit_3d uses
    return solvers, pf, alg, esp


def _quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def _crandn(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


# ------------------------------------------------------------------ solvers
def make_solvers(solvers, pf, alg):
    from oracle import solver_oracle as SO
    rng = np.random.RandomState(7)
    shape = (8, 8)
    N, M = 64, 96
    A = _crandn(rng, (M, N)) / np.sqrt(2 * M)
    xt = np.zeros(N, dtype=complex)
    xt[[3, 17, 30, 41, 58]] = [1.0, -0.6j, 0.8 + 0.2j, 0.5, -0.3]
    b = A @ xt + 0.01 * _crandn(rng, M)
    Q, _ = np.linalg.qr(_crandn(rng, (N, N)))
    x0 = _crandn(rng, shape) * 0.1

    Af = lambda x: A @ np.asarray(x).reshape(-1)                     # noqa: E731
    AHf = lambda y: (A.conj().T @ np.asarray(y)).reshape(shape)       # noqa: E731
    AAf = lambda x: AHf(Af(x))                                        # noqa: E731
    Tq = lambda x: (Q @ np.asarray(x).reshape(-1)).reshape(shape)     # noqa: E731
    iTq = lambda c: (Q.conj().T @ np.asarray(c).reshape(-1)).reshape(shape)   # noqa: E731
    Th = lambda x: SO.haar_dwt(x, 2, (0, 1))                          # noqa: E731
    iTh = lambda c: SO.haar_idwt(c, 2, (0, 1))                        # noqa: E731

    out = dict(A=A, b=b, Q=Q, x0=x0, shape=np.array(shape))
    nite, step, th = 12, 0.5, 0.05
    out["ist32_q"] = _quiet(solvers.IST_32, Af, AAf, AHf, Tq, iTq, b, nite, step, th)
    out["fist32_q"] = _quiet(solvers.FIST_32, Af, AAf, AHf, Tq, iTq, b, nite, step, th)
    out["ist32_haar"] = _quiet(solvers.IST_32, Af, AAf, AHf, Th, iTh, b, nite, step, th)
    out["fist32_haar"] = _quiet(solvers.FIST_32, Af, AAf, AHf, Th, iTh, b, nite, step, th)
    out["ist3_q"] = _quiet(solvers.IST_3, Af, AHf, Tq, iTq, b, nite, step, th)
    out["fist3_q"] = _quiet(solvers.FIST_3, Af, AHf, Tq, iTq, b, nite, step, th)
    out["ist2"] = _quiet(solvers.IST_2, Af, AHf, b, nite, step, th)
    out["fist2"] = _quiet(solvers.FIST_2, Af, AHf, b, nite, step, th)
    out["step"], out["th"], out["nite"] = step, th, nite

    rho = 1.5
    out["cgd"] = _quiet(pf.prox_l2_Afxnb_CGD, Af, AHf, b, x0, rho, 5)
    out["gd"] = _quiet(pf.prox_l2_Afxnb_GD, Af, AHf, b, x0, rho, 20, 0.05)
    out["admm_l1x"] = _quiet(solvers.ADMM_l2Afxnb_l1x, Af, AHf, b, 6, 1.0, 0.02, 1.0, 3)
    out["admm_l1x_2"] = _quiet(solvers.ADMM_l2Afxnb_l1x_2, Af, AHf, b, 6, 1.0, 0.02, 1.0, 3)
    out["admm_l1Tfx_q"] = _quiet(solvers.ADMM_l2Afxnb_l1Tfx, Af, AHf, Tq, iTq, b, 6, 1.0, 0.02, 1.0, 3)
    out["rho"] = rho

    v = _crandn(rng, shape)
    out["soft_in"] = v
    out["soft"] = pf.prox_l1_soft_thresh(v.copy(), 0.7)
    out["soft2"] = pf.prox_l1_soft_thresh2(v.copy(), 0.7)
    f = lambda xi: np.linalg.norm(Af(xi) - b) ** 2                   # noqa: E731
    df = lambda xi: 2 * AHf(Af(xi) - b)                               # noqa: E731
    p = -df(x0) * 3.0                                                 # a long step: several shrinks
    alpha, nls = alg.BacktrackingLineSearch(f, df, x0, p)
    out["ls_p"], out["ls_alpha"], out["ls_n"] = p, alpha, nls
    return out


# ------------------------------------------------------------------ ESPIRiT
def _coil_kspace(shape, nc, rng):
    """Smooth synthetic coil images of a blob phantom, centred k-space (FFTWnd.forward)."""
    grids = np.meshgrid(*[np.linspace(-1, 1, n) for n in shape], indexing="ij")
    r2 = sum(g ** 2 for g in grids)
    img = (r2 < 0.6).astype(float) * (1.0 + 0.3 * grids[0]) + 0.2 * (r2 < 0.15)
    maps = []
    for c in range(nc):
        ang = 2 * np.pi * c / nc
        cen = [0.7 * np.cos(ang), 0.7 * np.sin(ang)] + [0.3 * (-1) ** c] * (len(shape) - 2)
        d2 = sum((g - c0) ** 2 for g, c0 in zip(grids, cen))
        maps.append(np.exp(-d2 / 1.5) * np.exp(1j * (0.4 * c + 0.5 * grids[1])))
    S = np.stack(maps, axis=-1)
    S /= np.sqrt(np.sum(np.abs(S) ** 2, axis=-1, keepdims=True))
    x = img[..., None] * S
    axes = tuple(range(len(shape)))
    k = np.fft.ifftshift(np.fft.fftn(np.fft.fftshift(x, axes), axes=axes), axes)
    return k + 1e-3 * _crandn(rng, k.shape)


def _centre(k, n):
    sl = tuple(slice(m // 2 - n // 2, m // 2 - n // 2 + n) for m in k.shape[:-1])
    return np.ascontiguousarray(k[sl])


def make_espirit(esp):
    rng = np.random.RandomState(11)
    out = {}
    k2 = _coil_kspace((32, 32), 4, rng)
    xc2 = _centre(k2, 12)
    out["k2_crop"] = xc2
    out["k2_shape"] = np.array([32, 32, 4])
    for pb, pf in ((1, 1), (0, 2), (0, 3)):
        V, s = _quiet(esp.espirit_2d, xc2, (32, 32, 4), 150, (5, 5), pb, pf, 0.01, 0.2)
        out["e2_pb%d_pf%d_V" % (pb, pf)] = V
        out["e2_pb%d_pf%d_s" % (pb, pf)] = s
    k3 = _coil_kspace((16, 16, 16), 4, rng)
    xc3 = _centre(k3, 8)
    out["k3_crop"] = xc3
    out["k3_shape"] = np.array([16, 16, 16, 4])
    for pb, pf in ((1, 1), (0, 2)):
        V, s = _quiet(esp.espirit_3d, xc3, (16, 16, 16, 4), 150, (3, 3, 3), pb, pf, 0.01, 0.2)
        out["e3_pb%d_pf%d_V" % (pb, pf)] = V
        out["e3_pb%d_pf%d_s" % (pb, pf)] = s
    return out


def main():
    root = MG.reference_root()
    solvers, pf, alg, esp = load(root)
    for name, data in (("golden_solvers.npz", make_solvers(solvers, pf, alg)),
                       ("golden_espirit.npz", make_espirit(esp))):
        path = os.path.join(HERE, name)
        np.savez_compressed(path, **data)
        print("wrote", path, "keys:", len(data), "bytes:", os.path.getsize(path))


if __name__ == "__main__":
    main()
