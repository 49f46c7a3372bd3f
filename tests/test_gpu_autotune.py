"""GPU tests of the autotuner and of the launch shapes it chooses between:
Shan-Chen strip heights and solo thresholds change no result; the tuner
picks one of its candidates, persists its table as JSON and looks shapes up
by nearest size bucket; a server driven by a tuned table still returns each
request's result as computed alone with the same nodes per thread."""
import numpy as np
import pytest

from tests.cases import fields_of, rel_err
from tests.test_gpu_batch import make

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


@pytest.mark.parametrize("kind", ["sc_bgk_f32", "sc_bgk_f16"])
def test_sc_rows_change_no_result(tl, kind):
    out = []
    for rows in (8, 16, 32):
        f, _ = make(tl, kind)
        s = f()
        b = tl.Batch(graphs=True, sc_rows=rows)
        b.add(s)
        b.run(30)
        s.finish()
        b.close()
        out.append(fields_of(s.lb))
    for o in out[1:]:
        for k in ("f", "rho", "vel"):
            assert rel_err(o[k], out[0][k]) == 0.0, k


def test_autotuner_table(tl, tmp_path):
    path = str(tmp_path / "tune.json")
    t = tl.Autotuner(path=path, steps=5, warmup=1)
    r = tl.Request(0, 512, 128, "trt", 0.58, 10, storage="fp16s")
    V = t.nodes_per_thread(r.tune_key(), "fp16s", lambda V: r.build(tl, nodes_per_thread=V))
    assert V in (4, 8)
    assert len(t.trials) == 2
    V2, solo, rows = t.batch_shape("mix", lambda V: [tl.Request(i, 256 + 64 * i, 64, "bgk", 0.6, 10,
                                                                storage="fp16s").build(tl, nodes_per_thread=V)
                                                     for i in range(3)], "fp16s")
    assert V2 in (4, 8) and rows == 0 and solo >= 0
    t.save()
    u = tl.Autotuner(path=path)
    assert u.lookup(r.tune_key(), "V") == V
    # a request of another size takes the nearest tuned bucket of its kind
    other = tl.Request(1, 1024, 256, "trt", 0.58, 10, storage="fp16s")
    assert u.lookup(other.tune_key(), "V") == V
    assert u.lookup(tl.Request(2, 512, 128, "bgk", 0.58, 10, storage="fp16s").tune_key(), "V") is None
    assert u.batch_kwargs("mix") == {"solo_nodes": solo}


def test_server_with_tuned_table(tl):
    t = tl.Autotuner(steps=5, warmup=1)
    reqs = [tl.Request(0, 256, 64, "bgk", 0.56, 300, storage="fp16s"),
            tl.Request(1, 320, 80, "mrt", 0.58, 70, arrival=0.01, storage="fp16s")]
    for r in reqs:  # force the non-default nodes per thread
        t.table[r.tune_key()] = {"V": 8}
    t.table["served"] = {"solo_nodes": 1, "sc_rows": 0}
    server = tl.Server(tl, hbm_budget=8 << 30, graphs=True, slice_steps=32, keep_fields=True, autotuner=t)
    for r in reqs:
        server.submit(r)
    done = server.run()
    server.close()
    for r in done:
        s = tl.Request(r.rid, r.nx, r.ny, r.model, r.tau, r.steps, storage="fp16s").build(tl, nodes_per_thread=8)
        series = s.step(r.steps, forces=True).cpu().numpy()
        ref = {"rho": s.lb.rho.to_numpy(), "vel": s.lb.vel.to_numpy()}
        for k in ("rho", "vel"):
            assert rel_err(r.fields[k], ref[k]) <= 1e-3, (r.rid, k)
        assert np.abs(r.forces - series).max() <= 1e-3 * max(np.abs(series).max(), 1e-12)
