"""In-place (AA-pattern) fused step against the ping-pong fused step.

FusedSolver(..., in_place=True) keeps one population buffer and alternates
two phases whose nodes read and write the same nine locations; between runs
the buffer holds what the ping-pong state holds.  Both read, round and store
the same values, so every result must be equal to the bit: f, f2, rho, vel
and pressure after step(n), the drag/lift series, and a checkpointed run.
Run lengths cover both phases ending a run (n - 1 fused steps, odd and
even), every storage, both node widths, BGK/TRT/MRT, the power law, a body
force, and every non-Shan-Chen fixture of the reference's boundary kinds
(NEEM and open boundaries read neighbour populations through the read-site
gather)."""
import numpy as np
import pytest
import torch

from tests.cases import build_from_case, cylinder_channel, fields_of, fixture_names, load_fixture
from tests.test_gpu_lean import periodic_box

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def assert_same(sa, sb, what=""):
    fa, fb = fields_of(sa.lb), fields_of(sb.lb)
    for k in ("f", "f2", "rho", "vel", "pressure"):
        assert np.array_equal(bits(fa[k]), bits(fb[k])), f"{what}: {k} differs"


def pair(tl, build, **kw):
    a = tl.FusedSolver(*build(), **kw)
    b = tl.FusedSolver(*build(), in_place=True, **kw)
    return a, b


def cylinder(tl, model="bgk"):
    def build():
        mrt_s = [0.0, 1.64, 1.54, 0.0, 1.7, 0.0, 1.7, 1 / 0.56, 1 / 0.56] if model == "mrt" else None
        return cylinder_channel(tl, 301, 67, 6.7, 60.2, 33.0, 0.56, 0.05, model=model, mrt_s=mrt_s)
    return build


@pytest.mark.parametrize("storage,V", [("fp32", 4), ("fp32", 2), ("fp16s", 4), ("bf16s", 8), ("i16s", 4),
                                       ("i16s", 8)])
@pytest.mark.parametrize("n", [2, 9, 40])
def test_cylinder_in_place_equals_ping_pong(tl, storage, V, n):
    a, b = pair(tl, cylinder(tl), storage=storage, nodes_per_thread=V)
    assert len(b._state_buffers()) == 1 and len(a._state_buffers()) == 2
    a.step(n)
    b.step(n)
    assert_same(a, b, f"{storage} V={V} n={n}")


@pytest.mark.parametrize("model", ["trt", "mrt"])
def test_models_in_place(tl, model):
    a, b = pair(tl, cylinder(tl, model), storage="fp16s")
    a.step(31)
    b.step(31)
    assert_same(a, b, model)


@pytest.mark.parametrize("storage", ["fp32", "i16s"])
def test_power_law_contraction_in_place(tl, storage):
    from taichi_lbm.workloads import contraction_channel

    def build():
        return contraction_channel(tl, 256, 64, 16, n=1.5, model="trt")
    a, b = pair(tl, build, storage=storage)
    a.step(26)
    b.step(26)
    assert_same(a, b, storage)


@pytest.mark.parametrize("model", ["bgk", "trt", "mrt"])
def test_periodic_box_with_force_in_place(tl, model):
    def build():
        return periodic_box(tl, model, tl.NewtonianFluid(0.05), True)
    a, b = pair(tl, build, storage="fp32")
    a.step(17)
    b.step(17)
    assert_same(a, b, model)


def test_forces_and_checkpoint_in_place(tl, tmp_path):
    a, b = pair(tl, cylinder(tl), storage="fp32")
    fa = a.step(24, forces=True)
    fb = b.step(24, forces=True)
    assert torch.equal(fa, fb)
    assert_same(a, b, "forces")
    # resume an in-place run from a checkpoint taken after an odd run
    c = tl.FusedSolver(*cylinder(tl)(), in_place=True)
    c.begin()
    c.run(13)
    torch.save(c.checkpoint(), tmp_path / "ck.pt")
    c.run(20)
    c.finish()
    d = tl.FusedSolver(*cylinder(tl)(), in_place=True)
    d.restore(torch.load(tmp_path / "ck.pt", weights_only=False))
    d.run(20)
    d.finish()
    assert_same(c, d, "resume")


def test_fixtures_in_place(tl):
    """Every non-Shan-Chen fixture the fused step accepts, in place against
    ping-pong; the compositions the in-place checks refuse are listed."""
    ran, refused = [], []
    for name in fixture_names():
        meta, arrays = load_fixture(name)
        if meta.get("sc") or "ibm" in name or name.startswith("mc_"):
            continue
        try:
            a = tl.FusedSolver(*build_from_case(tl, meta, arrays)[:4])
        except tl.UnsupportedComposition:
            continue
        try:
            b = tl.FusedSolver(*build_from_case(tl, meta, arrays)[:4], in_place=True)
        except tl.UnsupportedComposition as e:
            refused.append((name, str(e)))
            continue
        a.step(8)
        b.step(8)
        assert_same(a, b, name)
        ran.append(name)
    print("in place:", ran, "refused:", refused)
    assert len(ran) >= 8
    assert all("in-place step" in why for _, why in refused)
