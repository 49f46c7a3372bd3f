"""GPU tests of the serving loop: requests that arrive while others run are
admitted into the running batch (continuous batching) within an HBM budget,
and every request's result (final fields and its drag/lift series) is the
same as running it alone through FusedSolver.step(n, forces=True).  A
request that diverges (here: one whose initial populations hold a NaN,
planted on the host) is evicted at a slice boundary without touching the
others, and its work is not counted."""
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


def poisoned_request(tl, *a, **kw):
    """A Request whose lattice starts with a NaN in one fluid node's
    populations (host-side fault injection: the run diverges at once)."""
    class Poisoned(tl.Request):
        def build(self, tl_, keep_init=False, nodes_per_thread=None):
            s = super().build(tl_, keep_init=keep_init, nodes_per_thread=nodes_per_thread)
            s.lb._f[1, self.ny // 2, self.nx // 2 + self.nx // 4] = float("nan")
            return s
    return Poisoned(*a, **kw)


@pytest.mark.parametrize("storage", ["fp16s", "i16s"])
def test_diverged_request_is_evicted(tl, storage):
    server = tl.Server(tl, hbm_budget=8 << 30, graphs=True, slice_steps=16, keep_fields=True)
    good = [tl.Request(0, 256, 64, "bgk", 0.56, 600, arrival=0.0, storage=storage),
            tl.Request(2, 192, 48, "trt", 0.6, 300, arrival=0.0, storage=storage)]
    bad = poisoned_request(tl, 1, 160, 40, "mrt", 0.58, 5000, arrival=0.0, storage=storage)
    for r in (good[0], bad, good[1]):
        server.submit(r)
    done = {r.rid: r for r in server.run()}
    server.close()
    assert sorted(done) == [0, 1, 2]
    b = done[1]
    assert b.failed and not b.finite
    assert b.steps_run < b.steps  # left the batch long before its step count
    for r in good:
        g = done[r.rid]
        assert g.failed is None and g.finite
        alone = tl.Request(r.rid, r.nx, r.ny, r.model, r.tau, r.steps, storage=storage)
        s = alone.build(tl)
        series = s.step(r.steps, forces=True).cpu().numpy()
        for k, ref in (("rho", s.lb.rho.to_numpy()), ("vel", s.lb.vel.to_numpy())):
            assert rel_err(g.fields[k], ref) <= 1e-3, (r.rid, k)
        assert np.abs(g.forces - series).max() <= 1e-3 * max(np.abs(series).max(), 1e-12)
    # only the finished requests' updates are counted
    assert server.lattice_updates == sum(r.updates for r in done.values() if r.failed is None)


def test_saturated_fixed_point_request_is_retried_coarser(tl):
    """A fixed-point request whose impulsive start leaves the default range
    (inlet peak 0.06: the stagnation pressure transient of population 0
    exceeds 1/16) is built again with a step twice as coarse and finishes;
    every request's result equals the same request run alone at the step it
    finished with."""
    server = tl.Server(tl, hbm_budget=8 << 30, graphs=True, slice_steps=16, keep_fields=True)
    reqs = [tl.Request(0, 300, 76, "bgk", 0.56, 400, arrival=0.0, umax=0.06, storage="i16s"),
            tl.Request(1, 256, 64, "trt", 0.6, 300, arrival=0.0, umax=0.02, storage="i16s")]
    for r in reqs:
        server.submit(r)
    done = {r.rid: r for r in server.run()}
    server.close()
    assert done[0].retries == 1 and done[0].fixed_exp == 18
    for q in reqs:
        r = done[q.rid]
        assert r.failed is None and r.finite
        alone = tl.Request(q.rid, q.nx, q.ny, q.model, q.tau, q.steps, umax=q.umax, storage="i16s",
                           fixed_exp=r.fixed_exp)
        s = alone.build(tl)
        series = s.step(alone.steps, forces=True).cpu().numpy()
        assert not s.saturated
        for k, ref in (("rho", s.lb.rho.to_numpy()), ("vel", s.lb.vel.to_numpy())):
            assert rel_err(r.fields[k], ref) <= 1e-5, (q.rid, k)
        assert np.abs(r.forces - series).max() <= 1e-5 * np.abs(series).max()
