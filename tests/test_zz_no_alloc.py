"""The allocation-free moment reduction, called through the C ABI.

lbm_plan_reduce_moments_noalloc serves callers that cannot allocate device
memory themselves (a host whose device memory all belongs to its own pool or
HBM budget, or a between-steps monitor that must not trigger cudaMalloc):
its partial sums live in a fixed device array inside the library.  It must
give the same FP64 sums as lbm_plan_reduce_moments, which uses caller
scratch, call after call.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def vp(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_reduction_equals_scratch_reduction(built):
    import taichi_lbm as tl
    from taichi_lbm import _capi
    from taichi_lbm.workloads import cylinder_channel
    lib = _capi.load()
    lb, me, coll, be = cylinder_channel(tl, 320, 96, 9.6, 64.0, 47.5, 0.6, 0.04, keep_init=False)
    solver = tl.FusedSolver(lb, me, coll, be)
    solver.begin()
    solver.run(7)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    scratch = torch.empty(int(lib.lbm_reduce_scratch_doubles()), dtype=torch.float64, device="cuda")
    ref = torch.empty(3, dtype=torch.float64, device="cuda")
    assert lib.lbm_plan_reduce_moments(solver._plan, vp(scratch), vp(ref), stream) == 0
    outs = []
    for _ in range(2):  # two calls in a row share the library's scratch
        out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.lbm_plan_reduce_moments_noalloc(solver._plan, vp(out), stream)
        assert rc == 0, _capi.last_error()
        outs.append(out.cpu().numpy())
    r = ref.cpu().numpy()
    solver.finish()
    assert r[0] > 0
    for o in outs:
        assert abs(o[0] - r[0]) / r[0] < 1e-12
        assert abs(o[1] - r[1]) < 1e-9 and abs(o[2] - r[2]) < 1e-9
    assert np.array_equal(outs[0], outs[1])


def test_noalloc_reduction_rejects_lattices_over_the_limit(built):
    """The size check reads the plan's descriptor only and comes first, so
    an over-limit plan is rejected before any buffer is looked at: the plan
    here is created and never bound, and nothing is launched."""
    from taichi_lbm import _capi
    lib = _capi.load()
    d = _capi.LbmPlanDesc()
    d.nx, d.ny, d.pitch = 8192, 4097, 8192  # 8192 * 4097 sites > 2048 * 16384
    d.model, d.storage, d.nodes_per_thread, d.tau = _capi.BGK, _capi.STORE_F32, 4, 0.6
    plan = ctypes.c_void_p()
    assert lib.lbm_plan_create(ctypes.byref(d), ctypes.byref(plan)) == 0
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    rc = lib.lbm_plan_reduce_moments_noalloc(plan, vp(out), None)
    assert rc == -1  # LBM_ERR_ARG
    assert "exceeds the allocation-free limit" in _capi.last_error()
    lib.lbm_plan_destroy(plan)
