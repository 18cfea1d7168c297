"""The solver and ESPIRiT restatements pinned to mripy's own outputs (CPU).

The fixtures (tests/golden/golden_solvers.npz, golden_espirit.npz) were made by
tests/golden/make_golden_solvers.py, which ran the reference functions themselves
(pics/CS_MRI_solvers_func.py, pics/proximal_func.py, pics/opt_alg.py,
espirit/espirit_func.py) on a dense 96 x 64 complex operator and on synthetic multi-coil
k-space.  Checked here against them:

* oracle/solver_oracle.py   ist / fista (the IST_32 / FIST_32 loops with the Haar prox),
                            the restatement the GPU solvers are tested against
* mripy_gb300.solvers       IST_32, FIST_32, IST_3, FIST_3, IST_2, FIST_2 (host loops for
                            operators the library does not run natively)
* mripy_gb300.admm          the ADMM solvers, l2 proxes and backtracking line search
* oracle/espirit_oracle.py  espirit (2-D and 3-D; maps up to one phase per pixel)

Tolerances: FP64 restatements of the same loops agree to rounding (1e-10 relative).
"""
import os

import numpy as np
import pytest

from mripy_gb300 import admm
from mripy_gb300 import solvers as S
from oracle import espirit_oracle as EO
from oracle import solver_oracle as SO

G = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-10


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture(scope="module")
def gs():
    return np.load(os.path.join(G, "golden_solvers.npz"))


@pytest.fixture(scope="module")
def ge():
    return np.load(os.path.join(G, "golden_espirit.npz"))


def _ops(g):
    A, Q = g["A"], g["Q"]
    shape = tuple(int(v) for v in g["shape"])
    Af = lambda x: A @ np.asarray(x).reshape(-1)                         # noqa: E731
    AHf = lambda y: (A.conj().T @ np.asarray(y)).reshape(shape)           # noqa: E731
    AAf = lambda x: AHf(Af(x))                                            # noqa: E731
    Tq = lambda x: (Q @ np.asarray(x).reshape(-1)).reshape(shape)         # noqa: E731
    iTq = lambda c: (Q.conj().T @ np.asarray(c).reshape(-1)).reshape(shape)   # noqa: E731
    return Af, AHf, AAf, Tq, iTq


# ------------------------------------------------------------------ IST / FISTA
def test_oracle_ist_fista_haar_match_reference(gs):
    Af, AHf, AAf, _, _ = _ops(gs)
    n, step, th = int(gs["nite"]), float(gs["step"]), float(gs["th"])
    rhs = AHf(gs["b"])
    assert rel(SO.ist(AAf, rhs, n, step, th, 2, (0, 1)), gs["ist32_haar"]) < TOL
    assert rel(SO.fista(AAf, rhs, n, step, th, 2, (0, 1)), gs["fist32_haar"]) < TOL


def test_package_host_loops_match_reference(gs):
    Af, AHf, AAf, Tq, iTq = _ops(gs)
    b = gs["b"]
    n, step, th = int(gs["nite"]), float(gs["step"]), float(gs["th"])
    Th = lambda x: SO.haar_dwt(x, 2, (0, 1))       # noqa: E731
    iTh = lambda c: SO.haar_idwt(c, 2, (0, 1))     # noqa: E731
    assert rel(S.IST_32(Af, AAf, AHf, Tq, iTq, b, n, step, th), gs["ist32_q"]) < TOL
    assert rel(S.FIST_32(Af, AAf, AHf, Tq, iTq, b, n, step, th), gs["fist32_q"]) < TOL
    assert rel(S.IST_32(Af, AAf, AHf, Th, iTh, b, n, step, th), gs["ist32_haar"]) < TOL
    assert rel(S.FIST_32(Af, AAf, AHf, Th, iTh, b, n, step, th), gs["fist32_haar"]) < TOL
    assert rel(S.IST_3(Af, AHf, Tq, iTq, b, n, step, th), gs["ist3_q"]) < TOL
    assert rel(S.FIST_3(Af, AHf, Tq, iTq, b, n, step, th), gs["fist3_q"]) < TOL
    assert rel(S.IST_2(Af, AHf, b, n, step, th), gs["ist2"]) < TOL
    assert rel(S.FIST_2(Af, AHf, b, n, step, th), gs["fist2"]) < TOL


def test_soft_thresholds_match_reference(gs):
    v = gs["soft_in"]
    assert rel(admm.prox_l1_soft_thresh(v.copy(), 0.7), gs["soft"]) < TOL
    assert rel(S.prox_l1_soft_thresh2(v.copy(), 0.7), gs["soft2"]) < TOL
    assert rel(SO.soft_thresh(v, 0.7), gs["soft2"]) < TOL


# ------------------------------------------------------------------ ADMM, l2 proxes, line search
def test_admm_and_l2_proxes_match_reference(gs):
    Af, AHf, _, Tq, iTq = _ops(gs)
    b, x0, rho = gs["b"], gs["x0"], float(gs["rho"])
    assert rel(admm.prox_l2_Afxnb_CGD(Af, AHf, b, x0, rho, 5), gs["cgd"]) < TOL
    assert rel(admm.prox_l2_Afxnb_GD(Af, AHf, b, x0, rho, 20, 0.05), gs["gd"]) < TOL
    assert rel(admm.ADMM_l2Afxnb_l1x(Af, AHf, b, 6, 1.0, 0.02, 1.0, 3), gs["admm_l1x"]) < TOL
    assert rel(admm.ADMM_l2Afxnb_l1x_2(Af, AHf, b, 6, 1.0, 0.02, 1.0, 3), gs["admm_l1x_2"]) < TOL
    assert rel(admm.ADMM_l2Afxnb_l1Tfx(Af, AHf, Tq, iTq, b, 6, 1.0, 0.02, 1.0, 3), gs["admm_l1Tfx_q"]) < TOL


def test_line_search_matches_reference(gs):
    Af, AHf, _, _, _ = _ops(gs)
    b, x0 = gs["b"], gs["x0"]
    f = lambda xi: np.linalg.norm(Af(xi) - b) ** 2      # noqa: E731
    df = lambda xi: 2 * AHf(Af(xi) - b)                  # noqa: E731
    alpha, n = admm.BacktrackingLineSearch(f, df, x0, gs["ls_p"])
    assert n == int(gs["ls_n"]) and n > 0
    assert alpha == pytest.approx(float(gs["ls_alpha"]), rel=1e-12)


# ------------------------------------------------------------------ ESPIRiT
def _phase_agreement(v, vr):
    """|<v, vr>| / (|v| |vr|) per pixel (1 = equal up to a phase)."""
    num = np.abs(np.sum(v * np.conj(vr), axis=-1))
    den = np.linalg.norm(v, axis=-1) * np.linalg.norm(vr, axis=-1)
    return num / np.maximum(den, 1e-300)


@pytest.mark.parametrize("case,win,resampled", [
    ("e2_pb1_pf1", (5, 5), False), ("e2_pb0_pf3", (5, 5), False), ("e2_pb0_pf2", (5, 5), True),
    ("e3_pb1_pf1", (3, 3, 3), False), ("e3_pb0_pf2", (3, 3, 3), False)])
def test_espirit_oracle_matches_reference(ge, case, win, resampled):
    d = len(win)
    key = "k2" if d == 2 else "k3"
    xcrop = ge[key + "_crop"]
    x_shape = tuple(int(v) for v in ge[key + "_shape"])
    pb, pf = (int(v) for v in case.split("_pb")[1].split("_pf"))
    V, s = EO.espirit(xcrop, x_shape, 150, win, pb, pf, 0.01, 0.2)
    Vr, sr = ge[case + "_V"], ge[case + "_s"]
    assert rel(s, sr) < 1e-9
    kept = np.linalg.norm(Vr, axis=-1) > 0
    assert np.array_equal(kept, np.linalg.norm(V, axis=-1) > 0)     # the same pixels thresholded
    if not resampled:
        agree = _phase_agreement(V[kept], Vr[kept])
        assert agree.min() > 1 - 1e-9
        assert rel(np.abs(V), np.abs(Vr)) < 1e-9
