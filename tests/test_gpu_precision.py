"""Precision of the storages against the FP64 oracle, and mass conservation.

Accuracy is max|a-b| / max|b| per field (rho, u) against the oracle run in
double precision.  The oracle is also run in single precision, the
reference's own arithmetic: its distance from the double run (the case's
"floor") is printed beside every result.  The bars are fixed:

* fp32 is at least as accurate as the reference's own fp32 arithmetic:
  err <= 1.5 x floor + 1e-6;
* the fixed-point storage (i16s, the 16-bit storage of the batched and
  served paths) is within 1e-3;
* fp16s and bf16s are recorded with loose ceilings (1e-2 and 0.2): their
  rounding of the stored deviations is biased in steady flow, and they miss
  1e-3 (measured 2.8e-3 to 9e-3 for fp16s).

Cases, all steady or slowly developing, so that the floor stays far below
the bars:

* the power-law contraction (taichi_lbm.workloads.contraction_channel, the
  reference's cases/contraction flow.py with a power-law fluid; TRT,
  relaxation time clamped to [0.505, 2.0], inlet peak 0.02) for n = 1.0 and
  1.5, 512 x 128 (outlet 32 high), 4,000 steps;
* the cylinder channel at Re = 20 (512 x 128, radius 12.8, inlet peak 0.04),
  10,000 steps.

The shear-thinning contraction (n = 0.5) is run and recorded without a bar:
its jet is unsteady at these resolutions, and the oracle's own fp32 run
differs from its FP64 run by 0.43 in u at 512 x 128 (9e-4 at 1024 x 256).
LBM_PRECISION_SIZE="nx,ny,outlet,steps" runs the contraction at another size
(the full configuration is "2048,512,128,20000").  Each case prints one JSON
line.

Mass: a closed periodic box (no inflow or outflow, so the exact mass is
constant) runs 10,000 fused steps; the FP64 reduction of the population sum
before and after gives the relative drift.  The fixed-point storage
conserves every node's stored sum exactly, so only the reduction's own
rounding remains (bar 1e-13, against 1e-10 per 10k steps asked of the
16-bit path); the floating-point storages drift as the reference's own fp32
arithmetic does (recorded, ceiling 1e-3).
"""
import json
import os
import warnings

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import describe, fields_of, rel_err
from tests.test_gpu_lean import periodic_box

pytestmark = pytest.mark.gpu

SIZE = tuple(int(v) for v in os.environ.get("LBM_PRECISION_SIZE", "512,128,32,4000").split(","))
STORAGES = ["fp32", "fp16s", "bf16s", "i16s"]
CEILING = {"fp16s": 1e-2, "bf16s": 0.2, "i16s": 1e-3}
DRIFT = {"fp32": 1e-3, "fp16s": 1e-3, "bf16s": 1e-3, "i16s": 1e-13}


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def contraction(tl, n, keep_init=False):
    from taichi_lbm.workloads import contraction_channel
    nx, ny, h, _ = SIZE
    return contraction_channel(tl, nx, ny, h, n=n, keep_init=keep_init)


def cylinder_re20(tl, keep_init=False):
    from taichi_lbm.workloads import cylinder_channel
    tau = 0.5 + 3.0 * 0.04 * 25.6 / 20.0  # Re = u_max D / nu = 20, D = 25.6
    return cylinder_channel(tl, 512, 128, 12.8, 102.4, 63.5, tau, 0.04, keep_init=keep_init)


CASES = {"contraction n=0.5": (lambda tl, k=False: contraction(tl, 0.5, k), "powerlaw", SIZE[3], False),
         "contraction n=1.0": (lambda tl, k=False: contraction(tl, 1.0, k), "powerlaw", SIZE[3], True),
         "contraction n=1.5": (lambda tl, k=False: contraction(tl, 1.5, k), "powerlaw", SIZE[3], True),
         "cylinder Re=20": (cylinder_re20, "standard", 10000, True)}

_refs = {}


def oracle_refs(tl, name):
    """(FP64 oracle fields, FP32 oracle fields) of a case, computed once."""
    if name not in _refs:
        build, kind, steps, _ = CASES[name]
        lb, me, coll, be = build(tl, True)
        meta, arrays = describe(lb, coll, be, steps, step_kind=kind, fp="f64")
        a64 = {k: (v.astype(np.float64) if v.dtype == np.float32 else v) for k, v in arrays.items()}
        _refs[name] = (O.replay(meta, a64), O.replay(dict(meta, fp="f32"), arrays))
    return _refs[name]


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("name", list(CASES))
def test_storage_vs_fp64(tl, name, storage):
    build, kind, steps, barred = CASES[name]
    lb, me, coll, be = build(tl)
    solver = tl.FusedSolver(lb, me, coll, be, storage=storage)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # the unbarred case may saturate; its status is printed
        solver.step(steps)
    got = fields_of(lb)
    ref64, ref32 = oracle_refs(tl, name)
    err = {k: rel_err(got[k], ref64[k]) for k in ("rho", "vel")}
    floor = {k: rel_err(ref32[k], ref64[k]) for k in ("rho", "vel")}
    print(json.dumps({"case": name, "nx": lb.NX, "ny": lb.NY, "steps": steps, "storage": storage,
                      "rel_err_rho": err["rho"], "rel_err_vel": err["vel"], "oracle_fp32_floor_rho": floor["rho"],
                      "oracle_fp32_floor_vel": floor["vel"], "status": solver.status_bits}))
    if not barred:
        return
    assert np.isfinite(got["rho"]).all() and solver.status_bits == 0
    for k in ("rho", "vel"):
        bar = 1.5 * floor[k] + 1e-6 if storage == "fp32" else CEILING[storage]
        assert err[k] <= bar, (k, err, floor)


@pytest.mark.parametrize("storage", STORAGES)
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
