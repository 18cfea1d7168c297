"""Solvers that call the NUFFT operators: CG-SENSE and mripy's IST/FISTA with a
wavelet soft-threshold (pics/CS_MRI_solvers_func.py, pics/proximal_func.py), on the GPU.

* ``cg_sense``      linear conjugate gradient on S^H A^H D A S x = S^H A^H D y; the normal
                    operator is the SENSE-fused type-21 pipeline, optionally replayed from a
                    CUDA graph; all scalars stay on the device (no host sync per iteration)
* ``IST_32``, ``FIST_32``, ``IST_wrap``, ``FIST_wrap``   mripy's iterations
                    (CS_MRI_solvers_func.py:75-86, 207-247) on torch CUDA tensors
* ``prox_l1_Tf_soft_thresh2``  soft threshold in a transform domain (proximal_func.py:46-52)
* ``DWTnd``         orthonormal multi-level Haar wavelet with the DWTnd interface
                    (pics/operators_class.py:394-416; backward = image -> coefficients)
"""
import math

import torch

__all__ = ["cg_sense", "IST_32", "FIST_32", "IST_wrap", "FIST_wrap", "prox_l1_Tf_soft_thresh2",
           "prox_l1_soft_thresh2", "DWTnd"]


def _vdot(a, b):
    return torch.sum(a.conj() * b)


def cg_sense(A, y, n_iter=20, x0=None, use_graph=True):
    """Solve (A^H A) x = A^H y for A = joint2operators(espirit, NUFFT) with ``n_iter``
    CG iterations.  ``A.forward_backward`` is the normal operator and ``A.backward(y)`` the
    right-hand side (both carry mripy's 1/M, which cancels).  Returns (x, residual norms)."""
    b = A.backward(y)
    if not isinstance(b, torch.Tensor):
        raise TypeError("cg_sense runs on torch CUDA tensors")
    shape = b.shape
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    xin = torch.empty_like(b)
    Ap = torch.empty_like(b)
    graph = None
    if use_graph:
        graph = A.normal_graph(xin.view((1,) + tuple(A.Bopt.im_shape)), Ap.view((1,) + tuple(A.Bopt.im_shape)))

    def normal(v):
        if graph is not None:
            xin.copy_(v)
            graph.launch()
            return Ap
        return A.forward_backward(v).reshape(shape)

    r = b - normal(x) if x0 is not None else b.clone()
    p = r.clone()
    rs = _vdot(r, r).real
    norms = []
    for _ in range(n_iter):
        q = normal(p)
        alpha = rs / _vdot(p, q).real
        x.add_(alpha * p)
        r.sub_(alpha * q)
        rs_new = _vdot(r, r).real
        p.mul_(rs_new / rs).add_(r)
        rs = rs_new
        norms.append(rs)
    if graph is not None:
        graph.close()
    return x, torch.stack(norms).sqrt()


# ---------------------------------------------------------------- proximal operators
def prox_l1_soft_thresh2(x0, th):
    a = x0.abs()
    return x0 / (a + 1e-6) * torch.clamp(a - th, min=0.0)


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
            print(float(torch.linalg.vector_norm(r)))
    return x


def FIST_32(Afunc, invAAfunc, invAfunc, Tfunc, invTfunc, b, Nite, step, th, verbose=False):
    invAb = invAfunc(b)
    y = step * invAb
    y_acc = torch.zeros_like(y)
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
            print(float(torch.linalg.vector_norm(r)))
    return x


def _wrap(solver, Aopt, Topt, b, Nite, step, th):
    Nite = 20 if Nite is None else Nite
    step = 0.1 if step is None else step
    th = 0.04 if th is None else th
    if Topt is None:
        class _Id:
            def forward(self, v):
                return v

            def backward(self, v):
                return v
        Topt = _Id()
    if not hasattr(Aopt, "forward_backward"):
        raise TypeError("the operator needs forward_backward (the *_32 solver forms)")
    return solver(Aopt.forward, Aopt.forward_backward, Aopt.backward, Topt.backward, Topt.forward, b, Nite, step,
                  th)


def IST_wrap(Aopt, Topt=None, b=None, Nite=None, step=None, th=None):
    return _wrap(IST_32, Aopt, Topt, b, Nite, step, th)


def FIST_wrap(Aopt, Topt=None, b=None, Nite=None, step=None, th=None):
    return _wrap(FIST_32, Aopt, Topt, b, Nite, step, th)


# ---------------------------------------------------------------- Haar wavelet
class DWTnd:
    """Orthonormal multi-level Haar transform over ``axes`` (sizes divisible by 2^level).

    backward(im) -> coefficient array of the same shape (approximation block first along
    every axis, details after, recursively: the layout of pywt.coeffs_to_array for Haar);
    forward(coeffs) -> image.  Any other wavelet name raises: only Haar is built."""

    def __init__(self, wavelet="haar", level=2, axes=(0, 1, 2)):
        if wavelet not in ("haar", "db1"):
            raise NotImplementedError("only the Haar wavelet is provided")
        self.wavelet = wavelet
        self.level = level
        self.axes = tuple(axes)
        self.shape = None

    @staticmethod
    def _fwd_axis(x, ax, n):
        idx_e = torch.arange(0, n, 2, device=x.device)
        sl = x.narrow(ax, 0, n)
        e = sl.index_select(ax, idx_e)
        o = sl.index_select(ax, idx_e + 1)
        s = 1.0 / math.sqrt(2.0)
        return torch.cat([(e + o) * s, (e - o) * s], dim=ax)

    @staticmethod
    def _inv_axis(x, ax, n):
        h = n // 2
        a = x.narrow(ax, 0, h)
        d = x.narrow(ax, h, h)
        s = 1.0 / math.sqrt(2.0)
        e, o = (a + d) * s, (a - d) * s
        st = torch.stack([e, o], dim=ax + 1)
        shp = list(a.shape)
        shp[ax] = n
        return st.reshape(shp)

    def backward(self, im):
        if self.shape is None:
            self.shape = tuple(im.shape)
        x = im.clone()
        sizes = [im.shape[a] for a in self.axes]
        for lv in range(self.level):
            n = [s >> lv for s in sizes]
            if any(v % 2 for v in n):
                raise ValueError("axis sizes must be divisible by 2^level")
            block = x
            for a, na in zip(self.axes, n):
                block = block.narrow(a, 0, na)
            y = block.clone()
            for a, na in zip(self.axes, n):
                y = self._fwd_axis(y, a, na)
            block.copy_(y)
        return x

    def forward(self, coeffs):
        x = coeffs.clone()
        sizes = [coeffs.shape[a] for a in self.axes]
        for lv in reversed(range(self.level)):
            n = [s >> lv for s in sizes]
            block = x
            for a, na in zip(self.axes, n):
                block = block.narrow(a, 0, na)
            y = block.clone()
            for a, na in zip(self.axes, n):
                y = self._inv_axis(y, a, na)
            block.copy_(y)
        return x
