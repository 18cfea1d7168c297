"""Auxiliary guarantees of the GPU path: run-to-run determinism of the spread and the
bounded-wait failure path, both without provoking any GPU fault.

* Determinism: without split tiles every output cell is summed by one thread in the
  samples' sorted order (stable radix sort), so two spreads of the same trajectory are
  bitwise equal; tiles shared by several work items merge with float atomics and are
  reproducible only to rounding.
* Bounded waits: gbn_plan_check_wait_expiry arms an mbarrier for bytes that no copy will
  deliver and lets the wait give up after a few probes; the plan's status word must then
  report GBN_ERR_TIMEOUT once and be clear afterwards, and the context must stay usable.
"""
import numpy as np
import pytest
import torch

from mripy_gb300._native import GbnError
from mripy_gb300.plan import NufftPlan, Tuning

pytestmark = pytest.mark.gpu

GBN_ERR_TIMEOUT = 8


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def cvec(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize("dim,shape,M,nc", [(2, (128, 96), 40000, 8), (3, (32, 32, 24), 30000, 4)])
def test_spread_bitwise_reproducible_without_split_tiles(dim, shape, M, nc):
    rng = np.random.default_rng(50 + dim)
    xs = [cuda(rng.uniform(-np.pi, np.pi, M)) for _ in range(dim)]
    # work items large enough that no tile is shared by two of them
    plan = NufftPlan(dim, shape, n_coil=nc, eps=5e-6, max_nspread=6 if dim == 3 else None,
                     tuning=Tuning(max_subproblem=1 << 20)).set_points(xs)
    assert plan.info()["split_tiles"] == 0
    c = cuda(cvec(rng, (M, nc)))
    g1 = plan.spread(c, grid=plan.grid()).clone()
    g2 = plan.spread(c, grid=plan.grid()).clone()
    assert torch.equal(g1, g2)
    i1 = plan.type1(c).clone()
    i2 = plan.type1(c).clone()
    assert torch.equal(i1, i2)
    plan.close()


def test_split_tiles_counted_and_reproducible_to_rounding():
    rng = np.random.default_rng(53)
    M, nc = 60000, 4
    xs = rng.uniform(-np.pi, np.pi, (2, M))
    xs[:, : M // 2] *= 0.03                       # a dense centre: its tiles split
    plan = NufftPlan(2, (96, 96), n_coil=nc, eps=5e-6).set_points([cuda(v) for v in xs])
    assert plan.info()["split_tiles"] > 0
    c = cuda(cvec(rng, (M, nc)))
    g1 = plan.spread(c, grid=plan.grid()).clone()
    g2 = plan.spread(c, grid=plan.grid()).clone()
    assert float((g1 - g2).norm() / g1.norm()) < 1e-6
    plan.close()


def test_bounded_wait_expiry_reports_timeout_and_clears():
    plan = NufftPlan(2, (32, 32), n_coil=1, eps=1e-3)
    plan.status()                                 # clean to begin with
    plan.check_wait_expiry(probes=64)
    with pytest.raises(GbnError) as err:
        plan.status()
    assert err.value.status == GBN_ERR_TIMEOUT
    plan.status()                                 # read once, then clear
    # the context is still usable: a transform on the same plan runs and reports no timeout
    rng = np.random.default_rng(54)
    plan.set_points([cuda(rng.uniform(-np.pi, np.pi, 500)), cuda(rng.uniform(-np.pi, np.pi, 500))])
    out = plan.type1(cuda(cvec(rng, (500, 1))))
    plan.status()
    assert torch.isfinite(torch.view_as_real(out)).all()
    with pytest.raises(GbnError):
        plan.check_wait_expiry(probes=0)          # outside 1 .. 65536: rejected, nothing launched
    plan.close()
