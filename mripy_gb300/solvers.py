"""Solvers that call the NUFFT operators: CG-SENSE and mripy's IST/FISTA with a
wavelet soft-threshold (pics/CS_MRI_solvers_func.py, pics/proximal_func.py).

* ``cg_sense``      linear CG on S^H A^H D A S x = S^H A^H D y.  With A a NUFFT operator or
                    joint2operators(espirit, NUFFT) the whole solve runs in the library
                    (gbn_cg_sense): per iteration the fused normal operator and three vector
                    kernels (FP64 inner products kept on the device) replayed as one CUDA
                    graph, no host synchronisation.  Other operators: the same algorithm
                    with torch vector ops around ``forward_backward``.
* ``IST_wrap``, ``FIST_wrap``   mripy's wrappers (CS_MRI_solvers_func.py:89-110, 227-247).
                    NUFFT / SENSE operators with T = DWTnd('haar') (or no T) run natively
                    (gbn_ista_haar: normal operator + one fused gradient-step / Haar prox /
                    momentum kernel per iteration, one graph); any other operator runs
                    ``IST_32`` / ``FIST_32`` (:75-86, 207-224) on its callables, or ``IST_3`` /
                    ``FIST_3`` (:63-73, 189-205) when it has no forward_backward.
* ``prox_l1_soft_thresh2``, ``prox_l1_Tf_soft_thresh2``   proximal_func.py:20-24, 46-52
* ``DWTnd``         DWTnd with the Haar wavelet (pics/operators_class.py:394-416; pywt's
                    wavedecn + coeffs_to_array layout, dwt/dwt_func.py:15-23) on the GPU
"""
import numpy as np
import torch

from . import plan as _plan

__all__ = ["cg_sense", "IST_32", "FIST_32", "IST_3", "FIST_3", "IST_2", "FIST_2", "IST_wrap", "FIST_wrap",
           "prox_l1_Tf_soft_thresh2", "prox_l1_soft_thresh2", "DWTnd"]


def _vdot(a, b):
    return torch.sum(a.conj() * b)


def _native_normal(A, rhs):
    """(plan, sens, dcf, vector shape) when A's normal operator runs in the library."""
    if hasattr(A, "normal_solver") and hasattr(A, "Bopt"):
        ns = A.normal_solver()
        if ns is None:
            return None
        p, s, dcf = ns
        return p, s, dcf, (1,) + tuple(A.Bopt.im_shape)
    if hasattr(A, "normal_solver") and hasattr(A, "im_shape"):
        trail = tuple(rhs.shape[A.dim:])
        nc = int(np.prod(trail)) if trail else 1
        p, s, dcf = A.normal_solver(nc)
        return p, s, dcf, (1,) + tuple(A.im_shape) + (nc,)
    return None


def _to_cuda(b):
    if isinstance(b, torch.Tensor):
        return b.to("cuda", torch.complex64), False
    return torch.from_numpy(np.ascontiguousarray(np.asarray(b).astype(np.complex64))).to("cuda"), True


def cg_sense(A, y, n_iter=20, x0=None, use_graph=True):
    """Solve (A^H A) x = A^H y with ``n_iter`` CG iterations; ``A.forward_backward`` is the
    normal operator and ``A.backward(y)`` the right-hand side (both carry mripy's 1/M,
    which cancels).  Returns (x, residual norms after every iteration)."""
    b = A.backward(y)
    if not isinstance(b, torch.Tensor):
        raise TypeError("cg_sense runs on torch CUDA tensors")
    nat = _native_normal(A, b)
    if nat is not None:
        p, s, dcf, vshape = nat
        rhs = b.reshape(vshape).contiguous()
        xs = None if x0 is None else x0.to("cuda", torch.complex64).reshape(vshape).contiguous()
        x, norms = p.cg(rhs, n_iter, sens=s, dcf=dcf, x0=xs, use_graph=use_graph)
        return x.reshape(b.shape), norms
    # any other operator: the same iteration around its forward_backward
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    r = b - A.forward_backward(x) if x0 is not None else b.clone()
    p = r.clone()
    rs = _vdot(r, r).real
    norms = []
    for _ in range(n_iter):
        q = A.forward_backward(p)
        alpha = rs / _vdot(p, q).real
        x.add_(alpha * p)
        r.sub_(alpha * q)
        rs_new = _vdot(r, r).real
        p.mul_(rs_new / rs).add_(r)
        rs = rs_new
        norms.append(rs)
    return x, torch.stack(norms).sqrt()


# ---------------------------------------------------------------- proximal operators
def prox_l1_soft_thresh2(x0, th):
    """x0 / (|x0| + 1e-6) * max(|x0| - th, 0) (proximal_func.py:20-24); CUDA complex64
    tensors go through the library's kernel."""
    if isinstance(x0, torch.Tensor) and x0.is_cuda and x0.dtype == torch.complex64 and x0.is_contiguous():
        return _plan.prox_haar(x0.reshape(-1), th, 0, (0,)).reshape(x0.shape)
    if isinstance(x0, torch.Tensor):
        a = x0.abs()
        return x0 / (a + 1e-6) * torch.clamp(a - th, min=0.0)
    a = np.abs(x0)
    return x0 / (a + 1e-6) * np.maximum(a - th, 0.0)


def prox_l1_Tf_soft_thresh2(Tfunc, invTfunc, x0, th):
    """argmin_x th*||T x||_1 + 1/2||x - x0||^2 for orthonormal T (proximal_func.py:46-52)."""
    return invTfunc(prox_l1_soft_thresh2(Tfunc(x0), th))


# ---------------------------------------------------------------- IST / FISTA
def IST_32(Afunc, invAAfunc, invAfunc, Tfunc, invTfunc, b, Nite, step, th, verbose=False):
    invAb = invAfunc(b)
    x_acc = step * invAb
    x = x_acc
    for _ in range(Nite):
        x = prox_l1_Tf_soft_thresh2(Tfunc, invTfunc, x_acc, th)
        r = invAAfunc(x) - invAb
        x_acc = x_acc - step * r
        if verbose:
            print(float(np.linalg.norm(np.asarray(r.cpu() if isinstance(r, torch.Tensor) else r))))
    return x


def FIST_32(Afunc, invAAfunc, invAfunc, Tfunc, invTfunc, b, Nite, step, th, verbose=False):
    invAb = invAfunc(b)
    y = step * invAb
    y_acc = y * 0
    x_pre = y
    t = [1.0] * (Nite + 1)
    x = y
    for k in range(Nite):
        r = invAAfunc(y) - invAb
        y_acc = y_acc - step * r
        x = prox_l1_Tf_soft_thresh2(Tfunc, invTfunc, y_acc, th)
        t[k + 1] = (1 + (1 + 4 * t[k] ** 2) ** 0.5) / 2
        y = x + ((t[k] - 1) / t[k + 1]) * (x - x_pre)
        x_pre = x
        if verbose:
            print(float(np.linalg.norm(np.asarray(r.cpu() if isinstance(r, torch.Tensor) else r))))
    return x


def IST_3(Afunc, invAfunc, Tfunc, invTfunc, b, Nite, step, th, verbose=False):
    """IST with the operator applied as forward and adjoint (CS_MRI_solvers_func.py:63-73):
    for operators without forward_backward."""
    x_acc = step * invAfunc(b)
    x = x_acc
    for _ in range(Nite):
        x = prox_l1_Tf_soft_thresh2(Tfunc, invTfunc, x_acc, th)
        r = Afunc(x) - b
        x_acc = x_acc - step * invAfunc(r)
        if verbose:
            print(float(np.linalg.norm(np.asarray(r.cpu() if isinstance(r, torch.Tensor) else r))))
    return x


def FIST_3(Afunc, invAfunc, Tfunc, invTfunc, b, Nite, step, th, verbose=False):
    """FISTA with the operator applied as forward and adjoint (CS_MRI_solvers_func.py:190-205)."""
    y = step * invAfunc(b)
    y_acc = y * 0
    x_pre = y
    t = [1.0] * (Nite + 1)
    x = y
    for k in range(Nite):
        r = Afunc(y) - b
        y_acc = y_acc - step * invAfunc(r)
        x = prox_l1_Tf_soft_thresh2(Tfunc, invTfunc, y_acc, th)
        t[k + 1] = (1 + (1 + 4 * t[k] ** 2) ** 0.5) / 2
        y = x + ((t[k] - 1) / t[k + 1]) * (x - x_pre)
        x_pre = x
        if verbose:
            print(float(np.linalg.norm(np.asarray(r.cpu() if isinstance(r, torch.Tensor) else r))))
    return x


class _Identity:
    def forward(self, v):
        return v

    def backward(self, v):
        return v


def IST_2(Afunc, invAfunc, b, Nite, step, th, verbose=False):
    """IST_3 without a transform (CS_MRI_solvers_func.py:29-40)."""
    T = _Identity()
    return IST_3(Afunc, invAfunc, T.backward, T.forward, b, Nite, step, th, verbose)


def FIST_2(Afunc, invAfunc, b, Nite, step, th, verbose=False):
    """FIST_3 without a transform (CS_MRI_solvers_func.py:151-166)."""
    T = _Identity()
    return FIST_3(Afunc, invAfunc, T.backward, T.forward, b, Nite, step, th, verbose)


def _haar_level(Topt, dim_axes):
    """Level of a Haar DWTnd over exactly the image axes, 0 for no transform, else None."""
    if Topt is None:
        return 0
    if isinstance(Topt, DWTnd) and tuple(a for a in Topt.axes) == tuple(dim_axes):
        return int(Topt.level)
    return None


def _wrap(fista, Aopt, Topt, b, Nite, step, th):
    Nite = 20 if Nite is None else Nite
    step = 0.1 if step is None else step
    th = 0.04 if th is None else th
    if not hasattr(Aopt, "forward_backward"):
        # the reference's *_3 / *_2 forms: forward and adjoint applied separately
        T = _Identity() if Topt is None else Topt
        solver = FIST_3 if fista else IST_3
        return solver(Aopt.forward, Aopt.backward, T.backward, T.forward, b, Nite, step, th)
    dim = getattr(getattr(Aopt, "Bopt", Aopt), "dim", None)
    native = (hasattr(Aopt, "normal_solver") and dim is not None and Nite >= 1
              and _haar_level(Topt, tuple(range(dim))) is not None
              and (isinstance(b, np.ndarray) or (isinstance(b, torch.Tensor) and b.is_cuda)))
    if native:
        bt, was_np = _to_cuda(b)
        invAb = Aopt.backward(bt)
        nat = _native_normal(Aopt, invAb)
        if nat is not None:
            p, s, dcf, vshape = nat
            level = _haar_level(Topt, tuple(range(dim)))
            x = p.ista(invAb.reshape(vshape).contiguous(), Nite, step, th, level, sens=s, dcf=dcf, fista=fista)
            x = x.reshape(invAb.shape)
            return x.cpu().numpy().astype(np.complex128) if was_np else x
    if Topt is None:
        Topt = _Identity()
    solver = FIST_32 if fista else IST_32
    return solver(Aopt.forward, Aopt.forward_backward, Aopt.backward, Topt.backward, Topt.forward, b, Nite, step,
                  th)


def IST_wrap(Aopt, Topt=None, b=None, Nite=None, step=None, th=None):
    return _wrap(False, Aopt, Topt, b, Nite, step, th)


def FIST_wrap(Aopt, Topt=None, b=None, Nite=None, step=None, th=None):
    return _wrap(True, Aopt, Topt, b, Nite, step, th)


# ---------------------------------------------------------------- Haar wavelet
class DWTnd:
    """Orthonormal multi-level Haar transform over ``axes`` (1 to 3 consecutive axes,
    sizes divisible by 2^level), computed by the library's tile kernel.

    backward(im) -> coefficient array of the same shape (pywt.coeffs_to_array layout:
    approximation block first along every axis, then the detail blocks of each level,
    coarsest first); forward(coeffs) -> image.  CUDA tensors stay on the GPU; numpy arrays
    and CPU tensors are copied to it and back.  Any other wavelet name raises: only Haar
    is built."""

    def __init__(self, wavelet="haar", level=2, axes=(0, 1, 2)):
        if wavelet not in ("haar", "db1"):
            raise NotImplementedError("only the Haar wavelet is provided")
        self.wavelet = wavelet
        self.level = level
        self.axes = tuple(axes)
        self.shape = None

    def _run(self, x, inverse):
        if isinstance(x, torch.Tensor):
            dev = x.device
            t = x.to("cuda", torch.complex64).contiguous()
            out = _plan.haar_dwt(t, self.level, self.axes, inverse=inverse)
            return out if dev.type == "cuda" else out.to(dev)
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(x).astype(np.complex64))).to("cuda")
        return _plan.haar_dwt(t, self.level, self.axes, inverse=inverse).cpu().numpy().astype(np.complex128)

    def backward(self, im):
        if self.shape is None:
            self.shape = tuple(im.shape)
        return self._run(im, False)

    def forward(self, coeffs):
        return self._run(coeffs, True)
