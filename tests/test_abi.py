"""The C-ABI library builds, loads and exports every entry point that include/gbnufft.h
declares; host-only entry points (parameters, status strings, error paths) behave.
No kernel is launched: these run without a GPU."""
import ctypes
import os
import re
import shutil
import subprocess

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


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of gbn_plan_desc, gbn_plan_info and gbn_layout have the header's
    fields in its order (read from the header) at its offsets and sizes (printed by a C
    program built against include/gbnufft.h)."""
    structs = {"gbn_plan_desc": N.PlanDesc, "gbn_plan_info": N.PlanInfo, "gbn_layout": N.Layout}
    # the field names, in order, from the header's struct definitions
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    for cname, cls in structs.items():
        body = re.search(r"typedef struct \{([^}]*)\}\s*" + cname + r"\s*;", text).group(1)
        names = [re.match(r"\w+", d.strip()).group(0)
                 for decl in body.split(";") if decl.strip()
                 for d in decl.split(None, 1)[1].split(",")]
        assert names == [f for f, _ in cls._fields_], cname
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gbnufft.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in cls._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {(ln.split()[0], ln.split()[1]): int(ln.split()[2]) for ln in out if ln.strip()}
    for cname, cls in structs.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


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


@pytest.mark.parametrize("field,value", [("spread_variant", 4), ("interp_variant", 3), ("fft_variant", 3),
                                         ("fft_variant", -1), ("coil_group", 3), ("threads", 100)])
def test_plan_create_rejects_bad_tuning_before_touching_the_device(field, value):
    """Out-of-range tuning fields are GBN_ERR_ARG, checked before any CUDA call (so the same
    with or without a GPU), and no plan is returned."""
    d = N.PlanDesc()
    d.dim, d.ms, d.mt, d.mu, d.eps, d.iflag, d.df, d.n_coil, d.n_traj = 3, 16, 16, 16, 5e-6, 1, 1.0, 1, 1
    d.max_nspread = 6
    setattr(d, field, value)
    h = ctypes.c_void_p()
    assert N.lib().gbn_plan_create(ctypes.byref(d), ctypes.byref(h)) == 1  # GBN_ERR_ARG
    assert field.split("_")[0] in N.last_error()
    assert not h.value


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
