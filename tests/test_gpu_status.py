"""The plan's device status word (LbmPlanBuffers.status, LBM_STATUS_* bits):
fixed-point saturation over colliding nodes only, non-finite populations,
and the async pipeline's bounded wait running out.

* A cylinder channel (inlet peak 0.03) in the fixed-point storage at the
  default step (2^-19, range 1/16) reports nothing: solid nodes (whose
  stored deviation -w_k rho_ref lies outside the range) and row padding are
  not checked.
* The same flow with fixed_exp = 22 (range 2^-7) leaves the range and is
  reported; a coarser step (fixed_exp = 18, range 1/8) covers it and stays
  within the fp32 run by the step's own rounding.
* A NaN planted in one node's populations (on the host, before the run) is
  reported as non-finite (floating-point storages) or saturated (fixed point).
* The async pipeline with a wait budget of one clock cycle: the first wait
  of every warp runs out before its copy lands, the warp waits for its
  copies in flight with the long budget and returns, finish() raises, and
  the next run on the same device is correct.
"""
import pytest
import torch

from tests.cases import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def cylinder(tl, umax=0.03):
    from taichi_lbm.workloads import cylinder_channel
    return cylinder_channel(tl, 301, 67, 6.7, 60.0, 33.0, 0.56, umax, keep_init=False)


def test_fixed_point_cylinder_reports_nothing(tl):
    lb, me, coll, be = cylinder(tl)
    s = tl.FusedSolver(lb, me, coll, be, storage="i16s")
    s.step(200)
    assert s.status_bits == 0 and not s.saturated


def test_fixed_point_range_and_saturation(tl):
    lb, me, coll, be = cylinder(tl)
    tl.FusedSolver(lb, me, coll, be, storage="fp32").step(200)
    want = {"rho": lb.rho.to_numpy(), "vel": lb.vel.to_numpy()}
    lb, me, coll, be = cylinder(tl)
    s = tl.FusedSolver(lb, me, coll, be, storage="i16s", fixed_exp=22)
    with pytest.warns(UserWarning, match="saturated"):
        s.step(200)
    assert s.saturated
    lb, me, coll, be = cylinder(tl)
    s = tl.FusedSolver(lb, me, coll, be, storage="i16s", fixed_exp=18)
    s.step(200)
    assert s.status_bits == 0
    for k in ("rho", "vel"):
        assert rel_err(getattr(lb, k).to_numpy(), want[k]) < 5e-3, k


@pytest.mark.parametrize("storage", ["fp32", "fp16s", "bf16s", "i16s"])
def test_nan_is_reported(tl, storage):
    lb, me, coll, be = cylinder(tl)
    lb._f[3, 30, 100] = float("nan")  # population 3 of node (100, 30), a fluid node
    s = tl.FusedSolver(lb, me, coll, be, storage=storage)
    with pytest.warns(UserWarning):
        s.step(20)
    want = tl._capi.STATUS_SATURATED if storage == "i16s" else tl._capi.STATUS_NONFINITE
    assert s.status_bits & want


def test_async_wait_expiry_is_reported_and_recoverable(tl):
    lb, me, coll, be = cylinder(tl)
    s = tl.FusedSolver(lb, me, coll, be, pipeline="async", wait_cycles=1)
    with pytest.raises(tl._capi.LbmError, match="time budget"):
        s.step(5)
    assert s.status_bits & tl._capi.STATUS_TIMEOUT
    torch.cuda.synchronize()
    # the device keeps working: with the default budget the async step agrees
    # with the direct one to fp32 rounding (the two collide with different
    # but equivalent instruction sequences)
    lb, me, coll, be = cylinder(tl)
    a = tl.FusedSolver(lb, me, coll, be, pipeline="async")
    a.step(30)
    assert a.status_bits == 0
    got = lb.f.to_numpy()
    lb, me, coll, be = cylinder(tl)
    tl.FusedSolver(lb, me, coll, be).step(30)
    assert rel_err(got, lb.f.to_numpy()) < 1e-5
