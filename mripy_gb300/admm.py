"""mripy's ADMM solvers and the proximal / line-search helpers they call, over any operator
given as callables (numpy arrays or torch tensors; with the NUFFT / SENSE operator classes
every A and A^H is the library's GPU pipeline):

* ``BacktrackingLineSearch``   pics/opt_alg.py:8-33 (Armijo backtracking, factor rho)
* ``prox_l1_soft_thresh``      pics/proximal_func.py:13-17 (exp(i angle(x)) max(|x| - th, 0))
* ``prox_l1_Tf_soft_thresh``   pics/proximal_func.py:38-44
* ``prox_l2_Afxnb_GD``         pics/proximal_func.py:240-254 (gradient descent)
* ``prox_l2_Afxnb_CGD``        pics/proximal_func.py:282-311 (Fletcher-Reeves nonlinear CG with
                               backtracking line search) for argmin ||A x - b||^2 + rho/2 ||x - x0||^2
* ``ADMM_l2Afxnb_l1x``         pics/CS_MRI_solvers_func.py:321-333
* ``ADMM_l2Afxnb_l1Tfx``       pics/CS_MRI_solvers_func.py:381-392
* ``ADMM_l2Afxnb_l1x_2``       pics/CS_MRI_solvers_func.py:437-451

The TV-regularised variants (ADMM_l2Afxnb_tvx, _tvTfx) need mripy's TV operators, which are
outside this library.  The reference prints a residual every iteration; here ``verbose``
does.
"""
import numpy as np
import torch

__all__ = ["BacktrackingLineSearch", "prox_l1_soft_thresh", "prox_l1_Tf_soft_thresh", "prox_l2_Afxnb_GD",
           "prox_l2_Afxnb_CGD", "ADMM_l2Afxnb_l1x", "ADMM_l2Afxnb_l1Tfx", "ADMM_l2Afxnb_l1x_2"]


def _norm(x):
    if isinstance(x, torch.Tensor):
        return float(torch.linalg.vector_norm(x))
    return float(np.linalg.norm(x))


def _re_vdot(a, b):
    """Re(sum a * conj(b)) -- the reference's np.real(np.dot(p.flatten(), np.conj(g).flatten()))"""
    if isinstance(a, torch.Tensor):
        return float(torch.sum(a * torch.conj(b)).real)
    return float(np.real(np.dot(np.ravel(a), np.conj(np.ravel(b)))))


def _zeros_like(x):
    return torch.zeros_like(x) if isinstance(x, torch.Tensor) else np.zeros(x.shape, dtype=x.dtype)


def BacktrackingLineSearch(f, df, x, p, c=0.0001, rho=0.2, ls_Nite=10):
    """Step alpha along direction p from x: shrink by rho until the Armijo condition holds or
    f stops increasing (opt_alg.py:8-33).  Returns (alpha, number of shrink steps)."""
    derphi = _re_vdot(p, df(x))
    f0 = f(x)
    alphak = 1.0
    f_try = f(x + alphak * p)
    i = 0
    while i < ls_Nite and f_try - f0 > c * alphak * derphi and f_try > f0:
        alphak = alphak * rho
        f_try = f(x + alphak * p)
        i += 1
    return alphak, i


def prox_l1_soft_thresh(x0, th):
    """exp(i angle(x0)) * max(|x0| - th, 0) (proximal_func.py:13-17)."""
    if isinstance(x0, torch.Tensor):
        return torch.sgn(x0) * torch.clamp(x0.abs() - th, min=0.0)
    a = np.abs(x0) - th
    a[a < 0] = 0
    return np.exp(1j * np.angle(x0)) * a


def prox_l1_Tf_soft_thresh(Tfunc, invTfunc, x0, th):
    """invT(soft(T x0, th)) with the exact-angle soft threshold (proximal_func.py:38-44)."""
    return invTfunc(prox_l1_soft_thresh(Tfunc(x0), th))


def prox_l2_Afxnb_GD(Afunc, invAfunc, b, x0, rho, Nite, step):
    """argmin_x ||A x - b||^2 + rho/2 ||x - x0||^2 by gradient descent (proximal_func.py:240-254)."""
    x = x0
    eps = 0.001
    r = -2 * invAfunc(-b) + rho * x0
    delta = _norm(r)
    delta0 = delta
    i = 0
    while i < Nite and delta > eps * delta0:
        r = -2 * invAfunc(Afunc(x) - b) - rho * (x - x0)
        x = x + step * r
        delta = _norm(r)
        i += 1
    return x


def prox_l2_Afxnb_CGD(Afunc, invAfunc, b, x0, rho, Nite, ls_Nite=10):
    """argmin_x ||A x - b||^2 + rho/2 ||x - x0||^2 by Fletcher-Reeves nonlinear CG with
    backtracking line search, starting from x0 (proximal_func.py:282-311)."""
    eps = 0.001
    i = 0

    def f(xi):
        return _norm(Afunc(xi) - b) ** 2 + (rho / 2) * _norm(xi - x0) ** 2

    def df(xi):
        return 2 * invAfunc(Afunc(xi) - b) + rho * (xi - x0)

    dx = -df(x0)
    alpha, nstp = BacktrackingLineSearch(f, df, x0, dx, ls_Nite=ls_Nite)
    x = x0 + alpha * dx
    s = dx
    delta0 = _norm(dx)
    deltanew = delta0
    while i < Nite and deltanew > eps * delta0 and nstp < ls_Nite:
        dx = -df(x)
        deltaold = deltanew
        deltanew = _norm(dx)
        beta = float(deltanew / float(deltaold))
        s = dx + beta * s
        alpha, nstp = BacktrackingLineSearch(f, df, x, s, ls_Nite=ls_Nite)
        x = x + alpha * s
        i += 1
    return x


def ADMM_l2Afxnb_l1x(Afunc, invAfunc, b, Nite, step, l1_r, rho, cgd_Nite=3, verbose=False):
    """argmin ||A x - b||^2 + l1_r ||x||_1 (CS_MRI_solvers_func.py:321-333)."""
    z = invAfunc(b)
    u = _zeros_like(z)
    x = z
    for _ in range(Nite):
        x = prox_l2_Afxnb_CGD(Afunc, invAfunc, b, z - u, rho, cgd_Nite)
        z = prox_l1_soft_thresh(x + u, l1_r / rho)
        u = u + step * (x - z)
        if verbose:
            print(_norm(x - z))
    return x


def ADMM_l2Afxnb_l1Tfx(Afunc, invAfunc, Tfunc, invTfunc, b, Nite, step, l1_r, rho, cgd_Nite=3, verbose=False):
    """argmin ||A x - b||^2 + l1_r ||T x||_1 (CS_MRI_solvers_func.py:381-392)."""
    z = invAfunc(b)
    u = _zeros_like(z)
    x = z
    for _ in range(Nite):
        x = prox_l2_Afxnb_CGD(Afunc, invAfunc, b, z - u, rho, cgd_Nite)
        z = prox_l1_Tf_soft_thresh(Tfunc, invTfunc, x + u, l1_r / rho)
        u = u + step * (x - z)
        if verbose:
            print("gradient in ADMM %g" % _norm(x - z))
    return x


def ADMM_l2Afxnb_l1x_2(Afunc, invAfunc, b, Nite, step, l1_r1, rho, cgd_Nite=3, verbose=False):
    """Consensus form with two copies of x (CS_MRI_solvers_func.py:437-451)."""
    z = invAfunc(b)
    u1 = _zeros_like(z)
    u2 = _zeros_like(z)
    x1 = z
    for _ in range(Nite):
        x1 = prox_l2_Afxnb_CGD(Afunc, invAfunc, b, z - u1, rho, cgd_Nite)
        x2 = prox_l1_soft_thresh(z - u2, l1_r1 / rho)
        z = (x1 + x2) / 2.0 + (u1 + u2) / 2.0
        u1 = u1 + step * (x1 - z)
        u2 = u2 + step * (x2 - z)
        if verbose:
            print(_norm(x2 - x1))
    return x1
