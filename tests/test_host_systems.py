"""Host-side logic of the batching and serving layers, without a GPU: the
autotuner's table (keys, nearest-bucket lookup, batch arguments, JSON round
trip), the serving loop's request stream and admission arithmetic, the
latency summary, and the replica timing of bench.py across two gloo ranks
(the max-over-ranks reduction the multi-GPU run uses)."""
import json
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from tests.cases import ROOT


def test_autotuner_keys_and_nearest_lookup(built, tmp_path):
    from taichi_lbm.autotune import Autotuner
    k = Autotuner.key("trt", "fp16s", 3000)
    assert k == "trt/fp16s/nt/plain/4096"
    assert Autotuner.key("bgk", "i16s", 4096, powerlaw=True) == "bgk/i16s/pl/plain/4096"
    t = Autotuner(path=str(tmp_path / "t.json"))
    t.table[Autotuner.key("trt", "fp16s", 1 << 14)] = {"V": 4}
    t.table[Autotuner.key("trt", "fp16s", 1 << 20)] = {"V": 8}
    t.table["served"] = {"solo_nodes": 0, "sc_rows": 16}
    # exact, nearest below, nearest above, other kind
    assert t.lookup(Autotuner.key("trt", "fp16s", 1 << 14), "V") == 4
    assert t.lookup(Autotuner.key("trt", "fp16s", 1 << 16), "V") == 4
    assert t.lookup(Autotuner.key("trt", "fp16s", 1 << 19), "V") == 8
    assert t.lookup(Autotuner.key("mrt", "fp16s", 1 << 14), "V") is None
    assert t.batch_kwargs("served") == {"solo_nodes": 0, "sc_rows": 16}
    assert t.batch_kwargs("absent") == {}
    t.save()
    u = Autotuner(path=str(tmp_path / "t.json"))
    assert u.table == json.loads(json.dumps(t.table))


def test_request_stream_is_seeded_and_in_range(built):
    from taichi_lbm.serving import request_stream
    a = request_stream(50, 10.0)
    b = request_stream(50, 10.0)
    assert [(r.nx, r.model, r.tau, r.steps, r.arrival) for r in a] == \
           [(r.nx, r.model, r.tau, r.steps, r.arrival) for r in b]
    for r in a:
        assert 128 <= r.nx <= 2048 and r.nx % 32 == 0 and r.ny == r.nx // 4
        assert r.model in ("bgk", "trt", "mrt")
        assert 0.5 < r.tau < 1.0 and 2000 <= r.steps <= 50000
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0)
    # the arrival process has about the requested rate (Poisson, 50 draws)
    assert 5.0 < 50 / arr[-1] < 20.0


def test_admission_bytes_grow_with_lattice_and_storage(built):
    from taichi_lbm.serving import device_bytes
    small, big = device_bytes(128, 32, "fp32"), device_bytes(2048, 512, "fp32")
    assert big > 200 * (small - (1 << 20))
    assert device_bytes(256, 64, "fp16s") > device_bytes(256, 64, "fp32")  # 16-bit state beside the fields
    # rows are padded to 32 elements
    assert device_bytes(129, 32, "fp32") == device_bytes(160, 32, "fp32")


def test_summary_percentiles(built):
    from taichi_lbm.serving import Request, summarize
    done = []
    for i, lat in enumerate([1.0, 2.0, 3.0, 4.0]):
        r = Request(i, 128, 32, "bgk", 0.6, 10, arrival=0.0)
        r.finished, r.finite = lat, i != 2
        done.append(r)
    s = summarize(done, 4.0, 8e6)
    assert s["requests"] == 4 and s["MLUPS"] == 2.0
    assert s["p50_s"] == 2.5 and s["finite"] == 3 and s["nonfinite_requests"] == [2]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica_rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    ms = [3.0, 5.0][rank]  # per-rank step time
    got = bench.max_over_ranks(ms, dist, device="cpu")
    out[rank] = got
    dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank():
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_replica_rank, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1] == 5.0


def test_ib_node_placement_matches_reference(built):
    """SphereIB / IBDEMCouplerEngine place the IB nodes and list the insiders
    exactly as the reference's ibm.py did for the immersed-circle fixture
    (host work; device tensors on the CPU here)."""
    import types
    from taichi_lbm.ibm import IBDEMCouplerEngine, IBEngine, SphereIB
    d = np.load(f"{ROOT}/tests/golden/ibm_circle_bgk_f32.npz")
    meta = json.loads(str(d["meta"]))
    ib = meta["ibm"]
    s = SphereIB(1, 64, device="cpu")
    c = np.array([ib["center"]])
    s.init_Balls(1, np.array([0]), c, np.zeros((1, 2)), np.zeros((1, 2)), np.zeros(1), np.array([ib["radius"]]),
                 np.zeros(1))
    s.init_IB_nodes()
    eng = IBDEMCouplerEngine(types.SimpleNamespace(NX=meta["NX"], NY=meta["NY"]))
    eng.SphereInfoUpdata(s, c, np.zeros((1, 2)), np.zeros(1))
    n = int(s.Sphere.NumIB[0])
    assert s.IBInsiderCount[None] == int(d["ib_count"]) == n
    assert np.array_equal(s.IBNodes.pos.to_numpy()[0, :n], d["ib_pos"])
    # ComputeParticleForce: the resultant is the last insider node's force
    f = np.zeros((1, 64, 2), np.float32)
    f[0, :n] = np.arange(2 * n, dtype=np.float32).reshape(n, 2)
    s.IBNodes.force.from_numpy(f)
    IBEngine(1).ComputeParticleForce(s)
    assert np.array_equal(s.Sphere.force.to_numpy()[0], f[0, n - 1])


def test_both_bench_arms_name_the_same_workload(built):
    """The reference arm's JSON line names the workload config of ours; its
    colliding-node count follows the disc rule of
    BoundaryEngine.Mask_cricle_identify (f32, strict)."""
    import types

    import bench
    import taichi_lbm as tl
    from taichi_lbm.fields import MaskField
    args = types.SimpleNamespace(nx=512, ny=128, model="bgk", storage="fp32", pipeline="direct", in_place=False,
                                 nodes_per_thread=None)
    cfg = bench.workload_config(args)
    n = bench.channel_active_nodes(cfg)
    owner = types.SimpleNamespace(NX=cfg["nx"], NY=cfg["ny"], mask=MaskField(cfg["nx"], cfg["ny"]))
    tl.BoundaryEngine().Mask_cricle_identify(owner, cfg["cx"], cfg["cy"], cfg["radius"])
    assert n == int((owner.mask.to_numpy() == 1).sum())
    ours = bench.arm_config(args, cfg, n, 4, 1)
    assert ours["updated_nodes_per_step"] == n and ours["nodes"] == 512 * 128
    assert ours["workload"].startswith("cylinder channel 512x128, r=12.5 at (100,64), BGK")
