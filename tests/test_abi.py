"""The C-ABI library builds, loads and exports every entry point that include/gbnufft.h
declares; host-only entry points (parameters, status strings, error paths) behave.
No kernel is launched: these run without a GPU."""
import ctypes
import os
import re

import pytest

from mripy_gb300 import _native as N
from mripy_gb300.plan import grid_params
import oracle as O

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "gbnufft.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbn_\w+)\s*\(", text)))


def test_header_and_binding_agree():
    assert header_functions() == sorted(N.EXPORTED)


def test_library_exports_every_declared_symbol():
    lib = N.lib()
    for name in header_functions():
        assert hasattr(lib, name), name
        assert getattr(lib, name) is not None


def test_version_and_status_strings():
    lib = N.lib()
    assert lib.gbn_version() >= 100
    assert lib.gbn_status_string(0) == b"ok"
    assert lib.gbn_status_string(1) == b"invalid argument"
    assert lib.gbn_status_string(99) == b"unknown status"


@pytest.mark.parametrize("dim,sizes,eps,clamp", [
    (1, (20, 1, 1), 5e-6, 0), (2, (128, 128, 1), 5e-6, 0), (2, (256, 256, 1), 1e-5, 0),
    (2, (15, 12, 1), 1e-3, 0), (2, (16, 16, 1), 1e-15, 0), (3, (8, 8, 6), 5e-6, 6),
    (3, (128, 128, 128), 5e-6, 6), (3, (8, 8, 6), 1e-12, 6), (3, (32, 32, 16), 0.05, 6),
])
def test_grid_params_match_oracle(dim, sizes, eps, clamp):
    ns, nf, tau = grid_params(dim, *sizes, eps=eps, max_nspread=clamp)
    ons, onf, otau = O.grid_params(dim, *sizes[:dim], eps=eps, max_nspread=clamp or None)
    assert ns == ons and nf == onf
    assert abs(tau - otau) <= 1e-15 * otau


def test_grid_params_rejects_bad_eps():
    with pytest.raises(N.GbnError) as ei:
        grid_params(2, 16, 16, eps=0.5)
    assert ei.value.status == 1
    assert "eps" in str(ei.value)


def test_null_arguments_are_rejected_without_touching_the_device():
    lib = N.lib()
    assert lib.gbn_plan_create(None, None) == 1
    assert lib.gbn_plan_destroy(None) == 0
    assert lib.gbn_graph_launch(None, None) == 1
    assert lib.gbn_type2(None, None, N.Layout(), None, N.Layout(), None) == 1
    buf = ctypes.create_string_buffer(64)
    assert lib.gbn_last_error(buf, 64) == 0
    assert buf.value  # message of the last failure


def test_plan_create_reports_missing_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    d = N.PlanDesc()
    d.dim, d.ms, d.mt, d.mu, d.eps, d.iflag, d.df, d.n_coil, d.n_traj = 2, 16, 16, 1, 1e-5, 1, 1.0, 1, 1
    h = ctypes.c_void_p()
    st = N.lib().gbn_plan_create(ctypes.byref(d), ctypes.byref(h))
    assert st == 3  # GBN_ERR_CUDA: no CUDA device, reported, not crashed
    assert "device" in N.last_error().lower()
    assert not h.value
