"""The oracle (FP64 restatement of mripy's CPU NUFFT) against golden vectors that
mripy's own code produced (tests/golden/make_golden.py).  CPU only."""
import os

import numpy as np
import pytest

import oracle as O

G = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-12  # FP64 restatement of the same loops: agreement to rounding


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.fixture(scope="module")
def g1():
    return np.load(os.path.join(G, "golden_1d.npz"))


@pytest.fixture(scope="module")
def g2():
    return np.load(os.path.join(G, "golden_2d.npz"))


@pytest.fixture(scope="module")
def g3():
    return np.load(os.path.join(G, "golden_3d.npz"))


def test_grid_params_match_reference_formula():
    # _compute_2d_grid_params(128, 128, 5e-6) -> (6, 256, 256, tau); eps 1e-5 -> nspread 5
    ns, nf, tau = O.grid_params(2, 128, 128, eps=5e-6)
    assert ns == 6 and nf == (256, 256)
    assert abs(tau - np.pi * 2.0 / 128 ** 2) < 1e-18
    assert O.grid_params(2, 16, 16, eps=1e-5)[0] == 5
    assert O.grid_params(2, 16, 16, eps=1e-15)[:2] == (14, (48, 48))   # function default: ratio 3
    assert O.grid_params(3, 8, 8, 6, eps=1e-12, max_nspread=6)[:2] == (6, (24, 24, 18))
    with pytest.raises(ValueError):
        O.grid_params(2, 16, 16, eps=0.5)


@pytest.mark.parametrize("eps,tag", [(5e-6, "e5em6"), (1e-3, "e1em3")])
@pytest.mark.parametrize("df", [1.0, 2.0])
@pytest.mark.parametrize("iflag", [1, -1])
def test_1d(g1, eps, tag, df, iflag):
    key = "%s_df%d_if%+d" % (tag, int(df), iflag)
    x, c, Fk = g1["x"], g1["c"], g1["Fk"]
    assert rel(O.nufft_type1((x,), c, (20,), df=df, eps=eps, iflag=iflag), g1["t1_" + key]) < TOL
    assert rel(O.nufft_type2((x,), Fk, (20,), df=df, eps=eps, iflag=iflag), g1["t2_" + key]) < TOL
    assert rel(O.nufft_type21((x,), Fk, (20,), df=df, eps=eps, iflag=iflag), g1["t21_" + key]) < TOL


@pytest.mark.parametrize("eps,tag", [(5e-6, "e5em6"), (1e-5, "e1em5")])
@pytest.mark.parametrize("df", [1.0, 2.0])
@pytest.mark.parametrize("iflag", [1, -1])
def test_2d_case_a(g2, eps, tag, df, iflag):
    key = "a_%s_df%d_if%+d" % (tag, int(df), iflag)
    x, y, c, Fk = g2["a_x"], g2["a_y"], g2["a_c"], g2["a_Fk"]
    assert rel(O.nufft_type1((x, y), c, (16, 16), df=df, eps=eps, iflag=iflag), g2["t1_" + key]) < TOL
    assert rel(O.nufft_type2((x, y), Fk, (16, 16), df=df, eps=eps, iflag=iflag), g2["t2_" + key]) < TOL
    assert rel(O.nufft_type21((x, y), Fk, (16, 16), df=df, eps=eps, iflag=iflag), g2["t21_" + key]) < TOL


@pytest.mark.parametrize("eps,tag", [(1e-5, "e1em5"), (1e-3, "e1em3")])
def test_2d_case_b_coils_odd_sizes(g2, eps, tag):
    key = "b_" + tag
    x, y, c, Fk = g2["b_x"], g2["b_y"], g2["b_c"], g2["b_Fk"]
    assert rel(O.nufft_type1((x, y), c, (15, 12), eps=eps), g2["t1_" + key]) < TOL
    assert rel(O.nufft_type2((x, y), Fk, (15, 12), eps=eps), g2["t2_" + key]) < TOL
    assert rel(O.nufft_type21((x, y), Fk, (15, 12), eps=eps), g2["t21_" + key]) < TOL


@pytest.mark.parametrize("eps,tag", [(5e-6, "e5em6"), (1e-5, "e1em5")])
@pytest.mark.parametrize("iflag", [1, -1])
def test_3d_case_a(g3, eps, tag, iflag):
    key = "a_%s_if%+d" % (tag, iflag)
    x, y, z, c, Fk, dcf = (g3[k] for k in ("a_x", "a_y", "a_z", "a_c", "a_Fk", "a_dcf"))
    s = (8, 8, 6)
    assert rel(O.nufft_type1((x, y, z), c, s, eps=eps, iflag=iflag), g3["t1_" + key]) < TOL
    assert rel(O.nufft_type2((x, y, z), Fk, s, eps=eps, iflag=iflag), g3["t2_" + key]) < TOL
    assert rel(O.nufft_type21((x, y, z), Fk, s, dcf=dcf, eps=eps, iflag=iflag), g3["t21_" + key]) < TOL


def test_3d_nspread_clamp(g3):
    x, y, z, c = (g3[k] for k in ("a_x", "a_y", "a_z", "a_c"))
    assert rel(O.nufft_type1((x, y, z), c, (8, 8, 6), eps=1e-12), g3["t1_a_e1em12_if+1"]) < TOL


def test_3d_operator_class(g3):
    op = O.NUFFT3dOracle(tuple(g3["b_shape"]), g3["b_dcf"])
    kx, ky, kz = op.normalize_set_ktraj(g3["b_ktraj"].copy())
    assert rel(kx, g3["b_kx"]) < TOL and rel(kz, g3["b_kz"]) < TOL
    assert rel(op.forward(g3["b_im"]), g3["b_forward"]) < TOL
    assert rel(op.backward(g3["b_kdata"]), g3["b_backward"]) < TOL
    assert rel(op.forward_backward(g3["b_im"]), g3["b_forward_backward"]) < TOL


def test_nudft_matches_reference_nudft(g1, g2, g3):
    assert rel(O.nudft_type1((g1["x"],), g1["c"], (20,)), g1["nudft1d1"]) < 1e-12
    assert rel(O.nudft_type1((g2["a_x"], g2["a_y"]), g2["a_c"], (16, 16)), g2["a_nudft2d1"]) < 1e-12
    assert rel(O.nudft_type1((g2["a_x"], g2["a_y"]), g2["a_c"], (16, 16), iflag=-1), g2["a_nudft2d1_if-1"]) < 1e-12
    assert rel(O.nudft_type1((g3["a_x"], g3["a_y"], g3["a_z"]), g3["a_c"], (8, 8, 6)), g3["a_nudft3d1"]) < 1e-12


def test_gridding_accuracy_vs_nudft():
    # nspread 6 (eps 5e-6) reaches ~1e-6 against the exact sum; nspread 3 only ~1e-3
    rng = np.random.default_rng(3)
    x, y = rng.uniform(-np.pi, np.pi, (2, 400))
    c = rng.standard_normal(400) + 1j * rng.standard_normal(400)
    F = rng.standard_normal((16, 16)) + 1j * rng.standard_normal((16, 16))
    assert rel(O.nufft_type1((x, y), c, (16, 16), eps=5e-6), O.nudft_type1((x, y), c, (16, 16))) < 1e-5
    assert rel(O.nufft_type2((x, y), F, (16, 16), eps=5e-6), O.nudft_type2((x, y), F, (16, 16))) < 1e-5
    assert rel(O.nufft_type1((x, y), c, (16, 16), eps=1e-3), O.nudft_type1((x, y), c, (16, 16))) > 1e-4


def test_adjointness_of_exact_sums():
    rng = np.random.default_rng(4)
    x, y = rng.uniform(-np.pi, np.pi, (2, 50))
    c = rng.standard_normal(50) + 1j * rng.standard_normal(50)
    F = rng.standard_normal((8, 6)) + 1j * rng.standard_normal((8, 6))
    lhs = np.vdot(c, O.nudft_type2((x, y), F, (8, 6)))
    rhs = 50 * np.vdot(O.nudft_type1((x, y), c, (8, 6)), F)
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)


def test_nudft_coordinate_gradient_finite_difference():
    rng = np.random.default_rng(5)
    x, y = rng.uniform(-np.pi, np.pi, (2, 20))
    F = rng.standard_normal((6, 6)) + 1j * rng.standard_normal((6, 6))
    gc = rng.standard_normal(20) + 1j * rng.standard_normal(20)
    g = O.nudft_type2_coord_grad((x, y), F, (6, 6), gc)
    h = 1e-6
    for j in (0, 7, 19):
        for d, arr in enumerate((x, y)):
            ap, am = arr.copy(), arr.copy()
            ap[j] += h
            am[j] -= h
            cp = O.nudft_type2((ap, y) if d == 0 else (x, ap), F, (6, 6))
            cm = O.nudft_type2((am, y) if d == 0 else (x, am), F, (6, 6))
            fd = np.real(np.vdot(gc, (cp - cm) / (2 * h)))
            assert abs(fd - g[j, d]) < 1e-6 * max(1.0, abs(fd))
