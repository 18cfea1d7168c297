"""mripy's ADMM solvers and their proximal / line-search helpers (mripy_gb300.admm) on a
dense operator, against a numpy restatement of the reference loops
(pics/CS_MRI_solvers_func.py:321-333, pics/proximal_func.py:282-311, pics/opt_alg.py:8-33).
CPU: the solvers are the operators' callers; the operators themselves are tested on the GPU."""
import numpy as np
import torch

from mripy_gb300 import admm


def _problem(seed=5):
    rng = np.random.default_rng(seed)
    A = (rng.standard_normal((48, 32)) + 1j * rng.standard_normal((48, 32))) / 8
    xt = np.zeros(32, dtype=complex)
    xt[[2, 9, 20]] = [1.0, -0.5j, 0.7]
    b = A @ xt + 0.01 * (rng.standard_normal(48) + 1j * rng.standard_normal(48))
    return A, b, xt


def _ls(f, df, x, p, c=0.0001, rho=0.2, ls_Nite=10):
    derphi = np.real(np.dot(p.flatten(), np.conj(df(x)).flatten()))
    f0 = f(x)
    a = 1.0
    ft = f(x + a * p)
    i = 0
    while i < ls_Nite and ft - f0 > c * a * derphi and ft > f0:
        a *= rho
        ft = f(x + a * p)
        i += 1
    return a, i


def _cgd(Af, AHf, b, x0, rho, Nite, ls_Nite=10):
    f = lambda xi: np.linalg.norm(Af(xi) - b) ** 2 + (rho / 2) * np.linalg.norm(xi - x0) ** 2  # noqa: E731
    df = lambda xi: 2 * AHf(Af(xi) - b) + rho * (xi - x0)                                        # noqa: E731
    dx = -df(x0)
    alpha, nstp = _ls(f, df, x0, dx, ls_Nite=ls_Nite)
    x = x0 + alpha * dx
    s = dx
    d0 = np.linalg.norm(dx)
    dn = d0
    i = 0
    while i < Nite and dn > 0.001 * d0 and nstp < ls_Nite:
        dx = -df(x)
        do, dn = dn, np.linalg.norm(dx)
        s = dx + (dn / do) * s
        alpha, nstp = _ls(f, df, x, s, ls_Nite=ls_Nite)
        x = x + alpha * s
        i += 1
    return x


def _soft(x0, th):
    a = np.abs(x0) - th
    a[a < 0] = 0
    return np.exp(1j * np.angle(x0)) * a


def test_admm_l1x_matches_reference_loop():
    A, b, xt = _problem()
    Af, AHf = (lambda v: A @ v), (lambda v: A.conj().T @ v)
    z = AHf(b)
    u = np.zeros_like(z)
    for _ in range(25):
        x = _cgd(Af, AHf, b, z - u, 1.0, 3)
        z = _soft(x + u, 0.05 / 1.0)
        u = u + 0.5 * (x - z)
    out = admm.ADMM_l2Afxnb_l1x(Af, AHf, b, 25, 0.5, 0.05, 1.0)
    assert np.allclose(out, x, atol=1e-10)
    assert np.linalg.norm(out - xt) < 0.2 * np.linalg.norm(xt)
    # torch tensors through the same code give the same iterate
    At = torch.from_numpy(A)
    outt = admm.ADMM_l2Afxnb_l1x(lambda v: At @ v, lambda v: At.conj().T @ v, torch.from_numpy(b), 25, 0.5, 0.05, 1.0)
    assert np.allclose(outt.numpy(), out, atol=1e-8)


def test_admm_variants_and_gradient_descent_prox():
    A, b, xt = _problem(6)
    Af, AHf = (lambda v: A @ v), (lambda v: A.conj().T @ v)
    ident = lambda v: v   # noqa: E731
    x1 = admm.ADMM_l2Afxnb_l1x(Af, AHf, b, 10, 0.5, 0.05, 1.0)
    x2 = admm.ADMM_l2Afxnb_l1Tfx(Af, AHf, ident, ident, b, 10, 0.5, 0.05, 1.0)
    assert np.allclose(x1, x2, atol=1e-12)           # T = identity reduces l1Tfx to l1x
    x3 = admm.ADMM_l2Afxnb_l1x_2(Af, AHf, b, 40, 0.5, 0.05, 1.0)
    assert np.linalg.norm(x3 - xt) < 0.3 * np.linalg.norm(xt)
    # the gradient-descent prox stops once its gradient fell by 1e-3, close to the minimiser;
    # the CG prox (beta = ||g_new|| / ||g_old||, as the reference has it) follows its loop exactly
    # and lowers the objective well below the start
    x0 = np.zeros(32, dtype=complex)
    g = admm.prox_l2_Afxnb_GD(Af, AHf, b, x0, 1.0, 2000, 0.05)
    ref = np.linalg.solve(2 * A.conj().T @ A + 1.0 * np.eye(32), 2 * A.conj().T @ b)
    assert np.linalg.norm(g - ref) < 1e-2 * np.linalg.norm(ref)
    c = admm.prox_l2_Afxnb_CGD(Af, AHf, b, x0, 1.0, 200)
    assert np.allclose(c, _cgd(Af, AHf, b, x0, 1.0, 200), atol=1e-12)
    obj = lambda v: np.linalg.norm(A @ v - b) ** 2 + 0.5 * np.linalg.norm(v) ** 2   # noqa: E731
    assert obj(c) < 0.25 * obj(x0) and obj(c) < 1.1 * obj(ref)


def test_line_search_shrinks_until_decrease():
    f = lambda x: float(np.sum(np.abs(x) ** 2))        # noqa: E731
    df = lambda x: 2 * x                               # noqa: E731
    x = np.array([1.0 + 0j])
    a, n = admm.BacktrackingLineSearch(f, df, x, -10 * df(x))
    assert n >= 1 and f(x + a * (-10 * df(x))) < f(x)
