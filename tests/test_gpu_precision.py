"""Precision of the storages against the FP64 oracle, and mass conservation.

Power-law contraction (taichi_lbm.workloads.contraction_channel, the
reference's cases/contraction flow.py with a power-law fluid, TRT, relaxation
time clamped to [0.505, 2.0], inlet peak 0.02): for n in {0.5, 1.0, 1.5} and
each storage, rho and u after N steps against the oracle run in double
precision.  Bounds: max|a-b|/max|b| per field <= 1e-4 for fp32, <= 1e-3 for
fp16-shifted, <= 1e-2 for bf16-shifted (8-bit significand).  The default
size is a 512 x 128 lattice (outlet 32 high) for 4,000 steps; with
LBM_PRECISION_FULL=1 the test runs the 2048 x 512 lattice (outlet 128 high)
for 20,000 steps instead.  Each case prints one JSON line with its errors.

Mass: a closed periodic box (no inflow or outflow, so the exact mass is
constant) runs 10,000 fused steps; the FP64 reduction of the population sum
before and after gives the relative drift, printed and bounded per storage.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import describe, fields_of, rel_err
from tests.test_gpu_lean import periodic_box

pytestmark = pytest.mark.gpu

FULL = os.environ.get("LBM_PRECISION_FULL") == "1"
SIZE = (2048, 512, 128, 20000) if FULL else (512, 128, 32, 4000)
TOL = {"fp32": 1e-4, "fp16s": 1e-3, "bf16s": 1e-2}
# relative mass drift over 10,000 steps of a 1024 x 1024 periodic box
DRIFT = {"fp32": 1e-10, "fp16s": 1e-6, "bf16s": 1e-4}


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


@pytest.fixture(scope="module")
def fp64_refs(tl):
    """FP64 oracle fields per power-law index, built once."""
    from taichi_lbm.workloads import contraction_channel
    nx, ny, h, steps = SIZE
    out = {}
    for n in (0.5, 1.0, 1.5):
        lb, me, coll, be = contraction_channel(tl, nx, ny, h, n=n, keep_init=True)
        meta, arrays = describe(lb, coll, be, steps, step_kind="powerlaw", fp="f64")
        arrays = {k: (v.astype(np.float64) if v.dtype == np.float32 else v) for k, v in arrays.items()}
        out[n] = O.replay(meta, arrays)
    return out


@pytest.mark.parametrize("storage", ["fp32", "fp16s", "bf16s"])
@pytest.mark.parametrize("n", [0.5, 1.0, 1.5])
def test_power_law_contraction_vs_fp64(tl, fp64_refs, n, storage):
    from taichi_lbm.workloads import contraction_channel
    nx, ny, h, steps = SIZE
    lb, me, coll, be = contraction_channel(tl, nx, ny, h, n=n)
    tl.FusedSolver(lb, me, coll, be, storage=storage).step(steps)
    got = fields_of(lb)
    ref = fp64_refs[n]
    err = {k: rel_err(got[k], ref[k]) for k in ("rho", "vel")}
    print(json.dumps({"case": "power-law contraction", "nx": nx, "ny": ny, "outlet": h, "steps": steps,
                      "n": n, "storage": storage, "rel_err_rho": err["rho"], "rel_err_vel": err["vel"]}))
    assert np.isfinite(got["rho"]).all()
    assert err["rho"] <= TOL[storage] and err["vel"] <= TOL[storage], err


@pytest.mark.parametrize("storage", ["fp32", "fp16s", "bf16s"])
def test_mass_drift_periodic_box(tl, storage):
    nx = ny = 1024
    lb, me, coll, be = periodic_box(tl, "bgk", tl.NewtonianFluid(0.05), False, nx=nx, ny=ny)
    s = tl.FusedSolver(lb, me, coll, be, storage=storage)
    s.begin()
    m0 = s.reduce_moments().cpu().numpy()
    s.run(10000)
    m1 = s.reduce_moments().cpu().numpy()
    s.finish()
    drift = abs(m1[0] - m0[0]) / abs(m0[0])
    print(json.dumps({"case": "mass drift, periodic box", "nx": nx, "ny": ny, "steps": 10000,
                      "storage": storage, "mass0": m0[0], "rel_drift": drift,
                      "momentum_drift": [float(m1[1] - m0[1]), float(m1[2] - m0[2])]}))
    assert drift <= DRIFT[storage], drift
