"""GPU tests of checkpoint/resume (FusedSolver.checkpoint / restore): a run
checkpointed part way, written to disk, and resumed by a solver built afresh
for the same lattice ends bit for bit where the uninterrupted run ends, for
fp32 and the shifted 16-bit storages, Newtonian and power law, Shan-Chen, and
for a member checkpointed inside a batch; a checkpoint does not load into
another lattice.
"""
import numpy as np
import pytest
import torch

from tests.cases import cylinder_channel, fields_of, rel_err
from tests.test_gpu_batch import make
from tests.test_gpu_lean import periodic_box

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def factory(tl, kind):
    if kind == "cyl_bgk_f32":
        def f():
            lb, me, coll, be = cylinder_channel(tl, 301, 67, 6.7, 60.2, 33.0, 0.56, 0.05)
            return tl.FusedSolver(lb, me, coll, be)
        return f
    if kind == "cyl_mrt_f16":
        def f():
            lb, me, coll, be = cylinder_channel(tl, 520, 64, 6.4, 104.0, 31.5, 0.56, 0.05, model="mrt",
                                                mrt_s=[0.0, 1.64, 1.54, 0.0, 1.7, 0.0, 1.7, 1 / 0.56, 1 / 0.56])
            return tl.FusedSolver(lb, me, coll, be, storage="fp16s")
        return f
    if kind == "box_trt_powerlaw_bf16":
        def f():
            lb, me, coll, be = periodic_box(tl, "trt", tl.PowerLawFluid(0.02, 0.7), True)
            return tl.FusedSolver(lb, me, coll, be, storage="bf16s")
        return f
    return make(tl, kind)[0]


@pytest.mark.parametrize("kind", ["cyl_bgk_f32", "cyl_mrt_f16", "box_trt_powerlaw_bf16", "sc_bgk_f16", "cyl_trt_i16"])
def test_resume_equals_uninterrupted(tl, kind, tmp_path):
    f = factory(tl, kind)
    a = f()
    a.begin()
    a.run(25)
    path = tmp_path / "ck.pt"
    torch.save(a.checkpoint(), path)
    a.run(30)
    a.finish()
    ref = fields_of(a.lb)

    b = f()
    b.restore(torch.load(path, weights_only=False))
    b.run(30)
    b.finish()
    got = fields_of(b.lb)
    for k in ("f", "f2", "rho", "vel"):
        assert rel_err(got[k], ref[k]) == 0.0, k
    assert b.lb.time[None] == a.lb.time[None]


def test_batch_member_checkpoint_resumes_alone(tl):
    """Checkpoint a member after batched steps; resuming it on its own gives
    the result of the member continuing in the batch."""
    fa = factory(tl, "cyl_mrt_f16")
    other = factory(tl, "cyl_bgk_f32")
    batch = tl.Batch(graphs=True)
    a, o = fa(), other()
    slot = batch.add(a)
    batch.add(o)
    batch.run(12)
    ck = a.checkpoint()
    batch.run(9)
    batch.remove(slot)
    a.finish()
    ref = fields_of(a.lb)
    b = fa()
    b.restore(ck)
    b.run(9)
    b.finish()
    got = fields_of(b.lb)
    for k in ("f", "rho", "vel"):
        assert rel_err(got[k], ref[k]) == 0.0, k
    o.finish()
    batch.close()


def test_checkpoint_rejects_other_lattice(tl):
    a = factory(tl, "cyl_bgk_f32")()
    a.begin()
    a.run(3)
    ck = a.checkpoint()
    a.finish()
    lb, me, coll, be = cylinder_channel(tl, 301, 67, 7.5, 60.2, 33.0, 0.56, 0.05)  # other cylinder
    b = tl.FusedSolver(lb, me, coll, be)
    with pytest.raises(ValueError):
        b.restore(ck)
    c = factory(tl, "cyl_bgk_f32")()
    with pytest.raises(RuntimeError):
        c.checkpoint()  # not live
    ck2 = dict(ck)
    ck2["format"] = "other"
    with pytest.raises(ValueError):
        c.restore(ck2)
    assert np.isfinite(fields_of(a.lb)["rho"]).all()
