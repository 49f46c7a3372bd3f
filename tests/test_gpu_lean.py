"""GPU parity of the two-pass direct step on lattices wide enough to have
interior row segments (x0 > 0 and the segment's right neighbour inside the
row), the case the lean kernel gathers without any wrap-around logic: every
collision model, fp32 and the shifted 16-bit storages, with and without a
body force, Newtonian and power law, against the oracle.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import cylinder_channel, describe, fields_of, rel_err
from tests.test_gpu_parity import TOL, TOL_PL, check_parity, fp64_solution

pytestmark = pytest.mark.gpu

# 520 columns: five 128-node segments at 4 nodes per lane, three of them interior
NX, NY = 520, 24
STORE_TOL = {"fp16s": 2e-3, "bf16s": 2e-2, "i16s": 2e-3}
MRT_S = [0.0, 1.64, 1.54, 0.0, 1.7, 0.0, 1.7, 1 / 0.65, 1 / 0.65]


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def periodic_box(tl, model, fluid, gravity, nx=NX, ny=NY, seed=7):
    """Fully periodic lattice with a random density and velocity field."""
    lb = tl.LBField("box", nx, ny, 1)
    lb.keep_init_snapshot = True
    cls = tl.BoundaryClassifier((nx, ny))
    be = tl.BoundaryEngine()
    fl = tl.FluidBoundary(spec=tl.BoundarySpec(geometry_fn=lambda i, j: lb.mask[i, j] == 1))
    fl.precompute(cls)
    be.add_boundary_condition("fluid", fl)
    per = tl.PeriodicAllBoundary(spec=tl.BoundarySpec(geometry_fn=lambda i, j: lb.mask[i, j] == 1))
    per.precompute(cls)
    be.add_boundary_condition("periodic", per)
    lb.neighbor_classify()
    me = tl.MacroscopicEngine(fl.group)
    params = {"group": fl.group, "fluid_model": fluid, "NX": nx, "NY": ny, "num_components": 1,
              "shearviscosity": [0.05]}
    if model == "bgk":
        coll = tl.BGKCollision(params)
    elif model == "trt":
        params["magic"] = [0.25]
        coll = tl.TRTCollision(params)
    else:
        params["bulkviscosity"] = [0.05]
        coll = tl.MRTCollision(params)
        if isinstance(fluid, tl.NewtonianFluid):
            coll.set_rates(MRT_S)
    rng = np.random.default_rng(seed)
    lb.rho.from_numpy((1 + 0.02 * rng.random((nx, ny, 1))).astype(np.float32))
    lb.vel.from_numpy((0.03 * (rng.random((nx, ny, 2)) - 0.5)).astype(np.float32))
    if gravity:
        lb.set_gravity([1e-5, -2e-5])
    lb.init_LBM(coll, fl.group)
    return lb, me, coll, be


def check_storage(got, ref64, storage):
    tol = STORE_TOL[storage]
    assert rel_err(got["rho"], ref64["rho"]) < tol
    assert rel_err(got["vel"], ref64["vel"]) < 10 * tol


@pytest.mark.parametrize("pipeline", ["direct", "prefetch"])
@pytest.mark.parametrize("gravity", [False, True])
@pytest.mark.parametrize("storage", ["fp32", "fp16s", "bf16s", "i16s"])
@pytest.mark.parametrize("model", ["bgk", "trt", "mrt"])
def test_lean_periodic_box(tl, model, storage, gravity, pipeline):
    lb, me, coll, be = periodic_box(tl, model, tl.NewtonianFluid(0.05), gravity)
    meta, arrays = describe(lb, coll, be, 120)
    solver = tl.FusedSolver(lb, me, coll, be, storage=storage, pipeline=pipeline)
    assert solver.nspecial == 0  # every segment takes the lean kernel
    solver.step(120)
    got = fields_of(lb)
    if storage == "fp32":
        check_parity(got, O.replay(meta, arrays), fp64_solution(meta, arrays), ("f", "rho", "vel"), TOL)
    else:
        check_storage(got, fp64_solution(meta, arrays), storage)


@pytest.mark.parametrize("pipeline", ["direct", "prefetch"])
@pytest.mark.parametrize("storage", ["fp32", "fp16s", "i16s"])
@pytest.mark.parametrize("model", ["bgk", "trt", "mrt"])
def test_lean_periodic_box_power_law(tl, model, storage, pipeline):
    lb, me, coll, be = periodic_box(tl, model, tl.PowerLawFluid(0.02, 0.7), True)
    meta, arrays = describe(lb, coll, be, 100, step_kind="powerlaw")
    tl.FusedSolver(lb, me, coll, be, storage=storage, pipeline=pipeline).step(100)
    got = fields_of(lb)
    if storage == "fp32":
        check_parity(got, O.replay(meta, arrays), fp64_solution(meta, arrays), ("f", "rho", "vel"), TOL_PL)
    else:
        check_storage(got, fp64_solution(meta, arrays), storage)


@pytest.mark.parametrize("storage", ["fp32", "fp16s", "i16s"])
@pytest.mark.parametrize("model", ["bgk", "trt", "mrt"])
def test_two_pass_forms_agree(tl, model, storage):
    """One general launch, the two launches serialised, and the two launches
    overlapped on the plan's side stream: the same step, on a channel with
    boundary segments (inlet, outlet, walls, cylinder) and interior ones."""
    s = MRT_S if model == "mrt" else None
    out = []
    for two_pass, overlap in ((False, False), (True, False), (True, True)):
        lb, me, coll, be = cylinder_channel(tl, NX, 64, 6.4, 104.0, 31.5, 0.56, 0.05, model=model, mrt_s=s)
        if not out:
            meta, arrays = describe(lb, coll, be, 150)
        solver = tl.FusedSolver(lb, me, coll, be, storage=storage, two_pass=two_pass, overlap=overlap)
        assert solver.launches_per_step == (2 if two_pass else 1)
        solver.step(150)
        out.append(fields_of(lb))
    tol = TOL if storage == "fp32" else STORE_TOL[storage]
    for k in ("rho", "vel"):
        assert rel_err(out[1][k], out[0][k]) < tol, k
        assert rel_err(out[2][k], out[1][k]) == 0.0, k  # same kernels, only the streams differ
    if storage == "fp32":
        check_parity(out[2], O.replay(meta, arrays), fp64_solution(meta, arrays), ("f", "rho", "vel"), TOL)
    else:
        check_storage(out[2], fp64_solution(meta, arrays), storage)


@pytest.mark.parametrize("tune", [0, 1, 2, 3])
@pytest.mark.parametrize("shape", [(520, 64), (389, 40)])
def test_prefetch_tunings_match_direct(tl, tune, shape):
    """Every shared-memory ring shape of the prefetching kernel gives the
    direct pipeline's result to the bit (same arithmetic, other loads); 389
    columns put node nx-1 inside a lane of a partial segment."""
    nx, ny = shape
    out = []
    for pipeline, t in (("direct", 0), ("prefetch", tune)):
        lb, me, coll, be = cylinder_channel(tl, nx, ny, ny / 10, nx / 5, ny / 2 - 0.5, 0.56, 0.05, model="trt")
        # both with per-segment special work (the prefetching form has no lane form)
        solver = tl.FusedSolver(lb, me, coll, be, storage="fp16s", pipeline=pipeline, tune=t,
                                lane_special=False)
        assert solver.launches_per_step == 2
        solver.step(60)
        out.append(fields_of(lb))
    for k in ("f", "f2", "rho", "vel"):
        assert rel_err(out[1][k], out[0][k]) == 0.0, k


@pytest.mark.parametrize("storage", ["fp32", "fp16s", "i16s"])
@pytest.mark.parametrize("shape", [(520, 64), (200, 48)])
def test_lane_special_equals_segment_special(tl, storage, shape):
    """Special work per lane (the plain kernel on every segment, one thread
    per marked lane) and per segment (the general kernel on every flagged
    segment) give the same step; 200 columns make most segments flagged."""
    nx, ny = shape
    out = []
    for lane_special in (False, True):
        lb, me, coll, be = cylinder_channel(tl, nx, ny, ny / 10, nx / 5, ny / 2 - 0.5, 0.56, 0.05, model="trt")
        solver = tl.FusedSolver(lb, me, coll, be, storage=storage, lane_special=lane_special)
        solver.step(80)
        out.append(fields_of(lb))
    tol = TOL if storage == "fp32" else STORE_TOL[storage]
    for k in ("rho", "vel"):
        assert rel_err(out[1][k], out[0][k]) <= tol, k
