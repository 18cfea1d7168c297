"""Host-side logic that needs no GPU: the wavelet class's argument check, proximal
operators, the IST/FISTA iterations on caller-supplied operators (checked against a numpy
restatement of mripy's loops), synthetic workloads, and the multi-rank timing reduction
of bench.py on two gloo processes."""
import math
import os
import socket

import numpy as np
import pytest
import torch

from mripy_gb300 import solvers, synth


def test_haar_rejects_other_wavelets():
    with pytest.raises(NotImplementedError):
        solvers.DWTnd("db2")


def test_soft_threshold_matches_reference_formula():
    rng = np.random.default_rng(0)
    x0 = rng.standard_normal(100) + 1j * rng.standard_normal(100)
    th = 0.7
    # proximal_func.py:20-24 (prox_l1_soft_thresh2)
    a = np.abs(x0) - th
    a[a < 0] = 0
    ref = x0 / (np.abs(x0) + 1e-6) * a
    out = solvers.prox_l1_soft_thresh2(torch.from_numpy(x0), th).numpy()
    assert np.allclose(out, ref, atol=1e-12)


class _DenseOp:
    def __init__(self, A):
        self.A = A

    def forward(self, x):
        return self.A @ x

    def backward(self, y):
        return self.A.conj().T @ y

    def forward_backward(self, x):
        return self.backward(self.forward(x))


def _fista_numpy(A, b, Nite, step, th):
    # numpy restatement of FIST_32 (CS_MRI_solvers_func.py:207-224) with T = identity
    invAb = A.conj().T @ b
    y = step * invAb
    y_acc = np.zeros_like(y)
    x_pre = y
    t = np.ones(Nite + 1)
    for k in range(Nite):
        r = A.conj().T @ (A @ y) - invAb
        y_acc = y_acc - step * r
        a = np.abs(y_acc) - th
        a[a < 0] = 0
        x = y_acc / (np.abs(y_acc) + 1e-6) * a
        t[k + 1] = (1 + (1 + 4 * t[k] ** 2) ** 0.5) / 2
        y = x + ((t[k] - 1) / t[k + 1]) * (x - x_pre)
        x_pre = x
    return x


def test_fista_matches_reference_loop():
    rng = np.random.default_rng(1)
    A = (rng.standard_normal((40, 30)) + 1j * rng.standard_normal((40, 30))) / 8
    b = rng.standard_normal(40) + 1j * rng.standard_normal(40)
    ref = _fista_numpy(A, b, 15, 0.5, 0.05)
    out = solvers.FIST_wrap(_DenseOp(torch.from_numpy(A)), None, torch.from_numpy(b), 15, 0.5, 0.05)
    assert np.allclose(out.numpy(), ref, atol=1e-10)


class _ForwardAdjointOp:
    """an operator without forward_backward: mripy's wrappers fall back to the *_3 forms"""
    def __init__(self, A):
        self.A = A

    def forward(self, x):
        return self.A @ x

    def backward(self, y):
        return self.A.conj().T @ y


def test_fista_without_forward_backward_matches_fist3_loop():
    rng = np.random.default_rng(4)
    A = (rng.standard_normal((40, 30)) + 1j * rng.standard_normal((40, 30))) / 8
    b = rng.standard_normal(40) + 1j * rng.standard_normal(40)
    # numpy restatement of FIST_3 (CS_MRI_solvers_func.py:189-205) with T = identity
    y = 0.5 * (A.conj().T @ b)
    y_acc = np.zeros_like(y)
    x_pre = y
    t = np.ones(16)
    for k in range(15):
        r = A @ y - b
        y_acc = y_acc - 0.5 * (A.conj().T @ r)
        a = np.abs(y_acc) - 0.05
        a[a < 0] = 0
        x = y_acc / (np.abs(y_acc) + 1e-6) * a
        t[k + 1] = (1 + (1 + 4 * t[k] ** 2) ** 0.5) / 2
        y = x + ((t[k] - 1) / t[k + 1]) * (x - x_pre)
        x_pre = x
    out = solvers.FIST_wrap(_ForwardAdjointOp(torch.from_numpy(A)), None, torch.from_numpy(b), 15, 0.5, 0.05)
    assert np.allclose(out.numpy(), x, atol=1e-10)
    out_ist = solvers.IST_wrap(_ForwardAdjointOp(A), None, b, 15, 0.5, 0.05)     # numpy in, numpy out
    assert isinstance(out_ist, np.ndarray)


def test_ist_decreases_objective():
    rng = np.random.default_rng(2)
    A = torch.from_numpy((rng.standard_normal((50, 20)) + 1j * rng.standard_normal((50, 20))) / 10)
    xt = torch.zeros(20, dtype=A.dtype)
    xt[[3, 11]] = 1.0
    b = A @ xt
    x = solvers.IST_wrap(_DenseOp(A), None, b, 200, 0.5, 1e-3)
    assert torch.linalg.vector_norm(x - xt) < 0.1


def test_synthetic_workloads():
    kx, ky = synth.radial_2d(128, 256)
    assert kx.shape == (32768,) and kx.min() >= -0.5 and kx.max() < 0.5
    kx, ky = synth.golden_radial_2d(402, 512)
    assert len(kx) == 402 * 512
    ang = math.atan2(ky[512 + 511], kx[512 + 511]) - math.atan2(ky[511], kx[511])
    assert abs(((ang + math.pi) % math.pi) - (synth.GOLDEN_ANGLE % math.pi)) < 1e-9
    S = synth.coil_maps((32, 24), 8)
    assert S.shape == (32, 24, 8)
    assert np.allclose(np.sum(np.abs(S) ** 2, axis=-1), 1.0, atol=1e-5)
    c3 = synth.config3()
    assert c3["spokes"].min() >= 5 and c3["spokes"].max() <= 34 and len(c3["offsets"]) == 65
    assert c3["offsets"][-1] == len(c3["k"][0]) == 384 * int(c3["spokes"].sum())
    k = synth.centre_out_radial_3d(100, 16)
    r = np.sqrt(k[0] ** 2 + k[1] ** 2 + k[2] ** 2)
    assert r.max() < 0.5 and len(k[0]) == 1600
    sx, sy = synth.vd_spiral_2d(24, 2048)
    assert len(sx) == 24 * 2048 and np.sqrt(sx ** 2 + sy ** 2).max() < 0.5


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    step_ms = 10.0 + 5.0 * rank                  # rank 1 is the slower replica
    mx = bench.max_over_ranks(step_ms)
    units = bench.replica_units(1000, world)
    q.put((rank, mx, units))
    dist.destroy_process_group()


def test_two_rank_gloo_timing_reduction():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]   # every rank sees the max step time
    assert [o[2] for o in out] == [2000, 2000]   # weak scaling: whole-job units = world * per-replica


def test_stencil_footprint_counts_cells_once():
    import bench
    nf, ns = (32, 32), 3
    one = bench.stencil_footprint([np.array([0.1]), np.array([6.2])], [0, 1], nf, ns)
    assert one == (2 * ns) ** 2                       # a stencil across the grid's edge wraps
    apart = bench.stencil_footprint([np.array([0.1, 3.0]), np.array([0.1, 3.0])], [0, 2], nf, ns)
    assert apart == 2 * (2 * ns) ** 2
    same = bench.stencil_footprint([np.array([0.1, 0.1]), np.array([0.1, 0.1])], [0, 2], nf, ns)
    assert same == (2 * ns) ** 2                      # overlapping stencils count once
    groups = bench.stencil_footprint([np.array([0.1, 0.1]), np.array([0.1, 0.1])], [0, 1, 2], nf, ns)
    assert groups == 2 * (2 * ns) ** 2                # but once per trajectory group
