"""GPU tests of the serving loop: requests that arrive while others run are
admitted into the running batch (continuous batching) within an HBM budget,
and every request's result (final fields and its drag/lift series) is the
same as running it alone through FusedSolver.step(n, forces=True)."""
import numpy as np
import pytest

from tests.cases import rel_err

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-5, "fp16s": 1e-3}


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def requests(tl, storage):
    """Request 0 runs long enough (thousands of steps) that the others,
    built by the builder thread meanwhile, join the batch while it runs."""
    R = tl.Request
    return [R(0, 256, 64, "bgk", 0.56, 6000, arrival=0.0, storage=storage),
            R(1, 160, 40, "trt", 0.60, 40, arrival=0.0, storage=storage),
            R(2, 320, 80, "mrt", 0.58, 70, arrival=0.02, storage=storage),
            R(3, 192, 48, "trt", 0.6, 55, arrival=0.03, powerlaw=(0.004, 0.8), storage=storage),
            R(4, 128, 32, "bgk", 0.62, 1, arrival=0.04, storage=storage)]


@pytest.mark.parametrize("storage", ["fp32", "fp16s"])
def test_served_results_equal_alone(tl, storage):
    server = tl.Server(tl, hbm_budget=8 << 30, graphs=True, slice_steps=16, keep_fields=True)
    for r in requests(tl, storage):
        server.submit(r)
    done = server.run()
    server.close()
    assert sorted(r.rid for r in done) == [0, 1, 2, 3, 4]
    overlapped = False
    for r in done:
        alone = tl.Request(r.rid, r.nx, r.ny, r.model, r.tau, r.steps, powerlaw=r.powerlaw, storage=storage)
        s = alone.build(tl)
        series = s.step(r.steps, forces=True).cpu().numpy()
        ref = {"rho": s.lb.rho.to_numpy(), "vel": s.lb.vel.to_numpy()}
        for k in ("rho", "vel"):
            assert rel_err(r.fields[k], ref[k]) <= TOL[storage], (r.rid, k)
        assert r.forces.shape == series.shape
        assert np.abs(r.forces - series).max() <= TOL[storage] * max(np.abs(series).max(), 1e-12), r.rid
        assert r.finite and r.latency is not None and r.latency >= 0
        overlapped |= any(o is not r and o.admitted < r.finished and r.admitted < o.finished for o in done)
    assert overlapped  # some requests shared the GPU


def test_admission_respects_budget(tl):
    """With room for one 256x64 lattice at a time the requests run one after
    another, in arrival order."""
    from taichi_lbm.serving import device_bytes
    budget = int(device_bytes(256, 64, "fp32") * 1.5)
    server = tl.Server(tl, hbm_budget=budget, graphs=False, slice_steps=8)
    for i in range(3):
        server.submit(tl.Request(i, 256, 64, "bgk", 0.6, 20, arrival=0.0, storage="fp32"))
    done = server.run()
    server.close()
    assert [r.rid for r in done] == [0, 1, 2]
    for a, b in zip(done, done[1:]):
        assert b.admitted >= a.finished - 1e-9
    with pytest.raises(ValueError):
        server.submit(tl.Request(9, 2048, 512, "bgk", 0.6, 10, storage="fp32"))
