"""GPU tests of batches (lbm_batch_*): every member's result in the mix equals
its result alone (FusedSolver.step on its own), whatever the mix of
collision models, storages, body forces, power law, Shan-Chen tiles and
lattice sizes; members may join and leave between runs (at either ping-pong
parity); graph replay equals direct launches; the batched drag/lift monitor
equals the per-lattice one; members run as solo single-lattice steps inside
the batch give the same results as packed ones.
"""
import numpy as np
import pytest

from tests.cases import cylinder_channel, fields_of, rel_err
from tests.test_gpu_lean import periodic_box

pytestmark = pytest.mark.gpu

MRT_S = [0.0, 1.64, 1.54, 0.0, 1.7, 0.0, 1.7, 1 / 0.56, 1 / 0.56]
# same kernels' arithmetic in both forms; the bound allows for a different
# fma contraction of the same expressions
TOL = {"fp32": 1e-5, "fp16s": 1e-3, "bf16s": 1e-2, "i16s": 1e-3}


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def make(tl, kind):
    """(solver factory, storage) for one member kind."""
    if kind == "cyl_bgk_f32":
        def f():
            lb, me, coll, be = cylinder_channel(tl, 301, 67, 6.7, 60.2, 33.0, 0.56, 0.05)
            return tl.FusedSolver(lb, me, coll, be)
        return f, "fp32"
    if kind == "cyl_trt_f16":
        def f():
            lb, me, coll, be = cylinder_channel(tl, 520, 64, 6.4, 104.0, 31.5, 0.56, 0.05, model="trt")
            return tl.FusedSolver(lb, me, coll, be, storage="fp16s")
        return f, "fp16s"
    if kind == "cyl_mrt_bf16":
        def f():
            lb, me, coll, be = cylinder_channel(tl, 256, 64, 6.4, 51.2, 31.5, 0.56, 0.05, model="mrt",
                                                mrt_s=MRT_S)
            return tl.FusedSolver(lb, me, coll, be, storage="bf16s")
        return f, "bf16s"
    if kind == "cyl_trt_i16":
        def f():
            lb, me, coll, be = cylinder_channel(tl, 416, 64, 6.4, 83.2, 31.5, 0.56, 0.05, model="trt")
            return tl.FusedSolver(lb, me, coll, be, storage="i16s", nodes_per_thread=8)
        return f, "i16s"
    if kind == "box_mrt_gravity_f32":
        def f():
            lb, me, coll, be = periodic_box(tl, "mrt", tl.NewtonianFluid(0.05), True, nx=389, ny=40)
            return tl.FusedSolver(lb, me, coll, be)
        return f, "fp32"
    if kind == "box_trt_powerlaw_f32":
        def f():
            lb, me, coll, be = periodic_box(tl, "trt", tl.PowerLawFluid(0.02, 0.7), True)
            return tl.FusedSolver(lb, me, coll, be)
        return f, "fp32"
    if kind == "box_bgk_v2_f32":
        def f():
            lb, me, coll, be = periodic_box(tl, "bgk", tl.NewtonianFluid(0.05), False)
            return tl.FusedSolver(lb, me, coll, be, nodes_per_thread=2)
        return f, "fp32"
    if kind == "sc_bgk_f32" or kind == "sc_bgk_f16":
        from taichi_lbm.workloads import carnahan_starling, shan_chen_box
        storage = "fp32" if kind.endswith("f32") else "fp16s"

        def f():
            rng = np.random.Generator(np.random.PCG64(11))
            psi, T = carnahan_starling(tl, 0.8)
            rho0 = 0.25 * (1.0 + rng.uniform(-0.01, 0.01, size=(200, 64)))
            lb, me, coll, be, sc, bsc = shan_chen_box(tl, 200, 64, psi, -1.0, T, rho0, model="bgk")
            return tl.FusedSolver(lb, me, coll, be, storage=storage, sc_boundary_engine=bsc)
        return f, storage
    raise KeyError(kind)


KINDS = ["cyl_bgk_f32", "cyl_trt_f16", "cyl_mrt_bf16", "cyl_trt_i16", "box_mrt_gravity_f32",
         "box_trt_powerlaw_f32", "box_bgk_v2_f32", "sc_bgk_f32", "sc_bgk_f16"]


def alone(tl, kind, n):
    factory, _ = make(tl, kind)
    s = factory()
    s.step(n)
    out = fields_of(s.lb)
    return out


def check_same(got, ref, storage, keys=("rho", "vel", "f")):
    for k in keys:
        assert rel_err(got[k], ref[k]) <= TOL[storage], (k, rel_err(got[k], ref[k]))


@pytest.mark.parametrize("solo", [None, 1])
@pytest.mark.parametrize("graphs", [False, True])
def test_mix_equals_alone(tl, graphs, solo):
    """solo=1: every member with special work runs its own single-lattice
    step inside the batched step instead of the packed tiles."""
    n = 40
    refs = {k: alone(tl, k, n) for k in KINDS}
    batch = tl.Batch(graphs=graphs, solo_nodes=solo)
    solvers = {}
    for k in KINDS:
        factory, _ = make(tl, k)
        solvers[k] = factory()
        batch.add(solvers[k])
    info = batch.info()
    batch.run(n - 1)
    info = batch.info()
    assert info["members"] == len(KINDS) and info["groups"] >= 6 and info["tiles"] > 0
    for k, s in solvers.items():
        s.finish()
        if s.sc is not None:
            s.lb.time[None] = s.lb.time[None] + n
        check_same(fields_of(s.lb), refs[k], make(tl, k)[1])
    batch.close()


def test_members_join_and_leave_at_either_parity(tl):
    """A runs 1 + 7 + 10 steps, B joins after 7 batched steps (opposite
    parity to the batch) and runs 1 + 10 + 5."""
    fa, _ = make(tl, "cyl_bgk_f32")
    fb, sb = make(tl, "cyl_trt_f16")
    ref_a = alone(tl, "cyl_bgk_f32", 18)
    ref_b = alone(tl, "cyl_trt_f16", 16)
    batch = tl.Batch(graphs=True)
    a = fa()
    slot_a = batch.add(a)
    batch.run(7)
    b = fb()
    batch.add(b)
    batch.run(10)
    batch.remove(slot_a)
    a.finish()
    batch.run(5)
    b.finish()
    check_same(fields_of(a.lb), ref_a, "fp32")
    check_same(fields_of(b.lb), ref_b, sb)
    batch.close()


def test_graph_replay_equals_direct_launches(tl):
    outs = []
    for graphs in (False, True):
        batch = tl.Batch(graphs=graphs)
        ss = []
        for k in ("cyl_bgk_f32", "cyl_trt_f16", "sc_bgk_f32"):
            s = make(tl, k)[0]()
            batch.add(s)
            ss.append(s)
        batch.run(9)  # odd: graph pairs plus direct steps
        batch.run(6)
        for s in ss:
            s.finish()
        outs.append([fields_of(s.lb) for s in ss])
        batch.close()
    for x, y in zip(outs[0], outs[1]):
        for k in ("f", "rho", "vel"):
            assert rel_err(x[k], y[k]) == 0.0, k


@pytest.mark.parametrize("solo", [None, 1])
def test_batched_monitor_equals_plan_series(tl, solo):
    n = 30
    lb, me, coll, be = cylinder_channel(tl, 200, 60, 6.0, 40.0, 29.5, 0.6, 0.05)
    ref = tl.FusedSolver(lb, me, coll, be).step(n, forces=True).cpu().numpy()
    batch = tl.Batch(graphs=True, solo_nodes=solo)
    lb, me, coll, be = cylinder_channel(tl, 200, 60, 6.0, 40.0, 29.5, 0.6, 0.05)
    s = tl.FusedSolver(lb, me, coll, be)
    other = make(tl, "cyl_trt_f16")[0]()
    slot = batch.add(s, monitor_steps=n)
    batch.add(other, monitor_steps=n)
    batch.run(n - 1)
    got = batch.forces(slot).cpu().numpy()
    s.finish()
    other.finish()
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    batch.close()


@pytest.mark.parametrize("form", [1, 2])
def test_lean_forms_equal_one_pass_form(tl, form):
    """The cp.async-pipelined forms of the packed plain segments
    (lbm_batch_set_lean_form 1 and 2) give every member the same populations
    as the one-pass form, to the bit (the gather and the collision are the
    same code; only where the source rows wait differs)."""
    n = 30
    kinds = [k for k in KINDS if not k.startswith("sc_")]
    out = {}
    for f in (0, form):
        batch = tl.Batch(graphs=True, solo_nodes=0, lean_form=f)
        solvers = {}
        for k in kinds:
            solvers[k] = make(tl, k)[0]()
            batch.add(solvers[k])
        batch.run(n - 1)
        for k, s in solvers.items():
            s.finish()
            out[(f, k)] = fields_of(s.lb)["f"]
        batch.close()
    for k in kinds:
        assert np.array_equal(out[(0, k)], out[(form, k)]), k
