"""Benchmark: MLUPS of the fused D2Q9 step on the 8192 x 2048 cylinder
channel (the roofline configuration), as a fraction of measured HBM
bandwidth, next to the CPU restatement of the reference timed on the host.

A "step" is one lattice-Boltzmann time step over the whole lattice.
  value  : lattice updates/s with the state resident in HBM (K fused steps)
  e2e    : the same through the drop-in API from host buffers: upload rho/u,
           init_LBM, FusedSolver.step(K), read rho/u back
  models : the other collision models and the 16-bit storages, same lattice; BGK fp32 and fp16s
           also in place (one population buffer, the AA pattern)
  batched: 64 periodic Shan-Chen lattices of uneven sizes in one Batch
  served : a Poisson stream of cylinder-channel requests through a Server,
           with p50/p99 latency, beside the same requests run alone in fp32
  --impl reference : the oracle (C++ restatement of taichi-lbm's unfused
           kernels, in the reference's call order) on the host cores

Multi-GPU: replicas only (independent lattices, no collective); value = sum
of all ranks' updates / max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

# more hardware queues than streams the batch and the server use (batch,
# workers, builders, retire), so independent streams never serialise; set
# before the CUDA context exists
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "taichi-lbm_gb300")
for _p in (PKG, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "MLUPS"
# algorithmic bytes per lattice update: 9 populations read + 9 written
BYTES_PER_LU = {"fp32": 72, "fp16s": 36, "bf16s": 36, "i16s": 36}
CONFIG = {"nx": 8192, "ny": 2048, "radius": 200.0, "cx": 1600.0, "cy": 1024.0, "tau": 0.52,
          "umax": 0.04}
MRT_S = [0.0, 1.64, 1.54, 0.0, 1.7, 0.0, 1.7, 1.0 / 0.52, 1.0 / 0.52]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--model", default="bgk", choices=["bgk", "trt", "mrt"])
    ap.add_argument("--storage", default="fp32", choices=["fp32", "fp16s", "bf16s", "i16s"])
    ap.add_argument("--nx", type=int, default=CONFIG["nx"])
    ap.add_argument("--ny", type=int, default=CONFIG["ny"])
    ap.add_argument("--nodes-per-thread", type=int, default=None)
    ap.add_argument("--pipeline", default="direct", choices=["direct", "async"])
    ap.add_argument("--in-place", action="store_true",
                    help="headline lattice on the in-place (AA-pattern) step, one population buffer")
    ap.add_argument("--no-extras", action="store_true", help="skip the per-model/storage lines")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched Shan-Chen lines")
    ap.add_argument("--no-served", action="store_true", help="skip the served request stream")
    ap.add_argument("--requests", type=int, default=256,
                    help="requests in the served stream (enough that the last requests' tail is a small part)")
    ap.add_argument("--served-capacity", type=float, default=None, metavar="MLUPS",
                    help="capacity the served stream's arrival rate is 80%% of (default: the single-lattice "
                         "BGK fp16s line)")
    ap.add_argument("--served-slice", type=int, default=200, help="steps per slice of the served batch")
    ap.add_argument("--served-shape", default=None, metavar="V,SOLO,FORM",
                    help="served batch shape (nodes per thread, solo threshold, lean form) instead of tuning it")
    ap.add_argument("--alone-sample", type=int, default=16,
                    help="served requests also run alone on the plain fp32 path, as the baseline")
    ap.add_argument("--mix-only", type=int, default=0, metavar="N",
                    help="only time the batched step of the first N served requests (all packed)")
    ap.add_argument("--mix-v", type=int, default=None, help="nodes per thread of the --mix-only members")
    ap.add_argument("--mix-form", type=int, default=0, choices=[0, 1, 2],
                    help="lean kernel form of the --mix-only batch (lbm_batch_set_lean_form)")
    ap.add_argument("--mix-storage", default="i16s", choices=["fp16s", "bf16s", "i16s"],
                    help="storage of the --mix-only members")
    ap.add_argument("--mix-solo", type=int, default=0, metavar="NODES",
                    help="--mix-only members of at least NODES nodes run their own step (0: all packed)")
    ap.add_argument("--mix-graphs", action="store_true", help="--mix-only batch replays CUDA graphs")
    ap.add_argument("--served-storage", default="i16s", choices=["fp32", "fp16s", "bf16s", "i16s"],
                    help="storage of the served requests")
    ap.add_argument("--batched-only", default=None, choices=["fp32", "fp16s", "bf16s"], metavar="STORAGE",
                    help="time only the batched Shan-Chen lattices in this storage")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    return ap.parse_args()


def workload_config(a):
    nx, ny = a.nx, a.ny
    s = nx / CONFIG["nx"]
    return {"nx": nx, "ny": ny, "radius": CONFIG["radius"] * s, "cx": CONFIG["cx"] * s,
            "cy": CONFIG["cy"] * ny / CONFIG["ny"], "tau": CONFIG["tau"], "umax": CONFIG["umax"]}


def arm_config(a, cfg, active, V, ws):
    """The workload both arms name in their JSON line (the reference arm
    times a bounded sample of it, described in its cpu_baseline)."""
    return {"workload": f"cylinder channel {cfg['nx']}x{cfg['ny']}, r={cfg['radius']:g} at "
                        f"({cfg['cx']:g},{cfg['cy']:g}), {a.model.upper()} tau={cfg['tau']}, "
                        f"parabolic inlet u_max={cfg['umax']}, PressureNEEM outlet, "
                        "bounce-back walls", "nodes": cfg["nx"] * cfg["ny"],
            "updated_nodes_per_step": int(active), "model": a.model, "storage": a.storage,
            "nodes_per_thread": int(V), "pipeline": a.pipeline, "in_place": a.in_place,
            "parallelism": f"replicas x{ws}",
            "l2": ("state (9 populations, one buffer)" if a.in_place else "state (2 x 9 populations)")
                  + " larger than L2; no flush needed"}


def channel_active_nodes(cfg):
    """Colliding nodes of the channel: every node outside the strict disc,
    in the f32 arithmetic of BoundaryEngine.Mask_cricle_identify."""
    import numpy as np
    x, y, r = np.float32(cfg["cx"]), np.float32(cfg["cy"]), np.float32(cfg["radius"])
    dx = np.arange(cfg["nx"], dtype=np.float32)[:, None] - x
    dy = np.arange(cfg["ny"], dtype=np.float32)[None, :] - y
    return int(cfg["nx"] * cfg["ny"] - np.count_nonzero((dx * dx + dy * dy) < (r * r)))


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(model, storage):
    """dram bytes per launch of the fused kernel from the committed ncu
    summary (profiles/), scaled to the full lattice there; None if absent."""
    path = os.path.join(ROOT, "profiles", f"fused_{model}_{storage}_cylinder.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch_full_lattice:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class Clocks:
    """Samples nvidia-smi every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": smax, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- GPU arm
def dist_setup():
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist
        rank = int(os.environ["RANK"])
        local = int(os.environ.get("LOCAL_RANK", rank))
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return rank, ws, local, dist
    torch.cuda.set_device(0)
    return 0, 1, 0, None


def max_over_ranks(v, dist, device="cuda"):
    """The slowest rank's value (replicas are timed by the slowest)."""
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    import torch
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
        torch.cuda.synchronize()


def build(tl, cfg, model, storage, V, pipeline="direct", in_place=False):
    from taichi_lbm.workloads import cylinder_channel
    lb, me, coll, be = cylinder_channel(tl, cfg["nx"], cfg["ny"], cfg["radius"], cfg["cx"], cfg["cy"],
                                        cfg["tau"], cfg["umax"], model=model,
                                        mrt_s=MRT_S if model == "mrt" else None, keep_init=False)
    solver = tl.FusedSolver(lb, me, coll, be, storage=storage, nodes_per_thread=V, pipeline=pipeline,
                            in_place=in_place)
    return lb, me, coll, be, solver


def time_resident(solver, K, W, dist, gpu_index):
    """K fused launches on the resident state, CUDA events on the launching stream."""
    import torch
    solver.begin()
    solver.run(W)
    barrier(dist)
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(gpu_index) as clk:
        barrier(dist)
        e0.record(s)
        solver.run(K)
        e1.record(s)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    barrier(dist)
    solver.finish()
    return ms, clk.summary()


def time_e2e(lb, coll, solver, K, dist):
    """Drop-in API from host buffers: pinned rho/u upload, init_LBM, step(K),
    rho/u download; host wall clock with device syncs on both sides."""
    import torch
    nx, ny = lb.NX, lb.NY
    active = coll.group.nodes
    rho0 = torch.zeros((nx, ny, 1), dtype=torch.float32).pin_memory()
    rho0[active[:, 0], active[:, 1], 0] = 1.0
    vel0 = torch.zeros((nx, ny, 2), dtype=torch.float32).pin_memory()
    rho_out = torch.empty_like(rho0).pin_memory()
    vel_out = torch.empty_like(vel0).pin_memory()
    barrier(dist)
    t0 = time.perf_counter()
    lb.rho.from_torch(rho0)
    lb.vel.from_torch(vel0)
    lb.init_LBM(coll, coll.group)
    solver.step(K)
    rho_out.copy_(lb.rho.to_torch(), non_blocking=True)
    vel_out.copy_(lb.vel.to_torch(), non_blocking=True)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    barrier(dist)
    if not torch.isfinite(rho_out).all():
        raise RuntimeError("non-finite density after the e2e run")
    h2d = rho0.numel() * 4 + vel0.numel() * 4
    d2h = rho_out.numel() * 4 + vel_out.numel() * 4
    return dt, h2d, d2h


def run_batched(tl, storage, K, W, gpu_index, graphs=True):
    """64 periodic Shan-Chen lattices of uneven sizes advanced together by one
    Batch: one persistent launch per step (a CUDA graph replays two steps).
    Returns aggregate MLUPS over every lattice and the roofline figures."""
    import torch
    from taichi_lbm.workloads import batched_shan_chen
    t0 = time.perf_counter()
    cases = batched_shan_chen(tl)
    solvers = [tl.FusedSolver(lb, me, coll, be, storage=storage, sc_boundary_engine=bsc)
               for lb, me, coll, be, sc, bsc in cases]
    nodes = sum(c[0].NX * c[0].NY for c in cases)
    setup = time.perf_counter() - t0
    # autotune the strip height (Shan-Chen plans run 4 nodes per thread) on
    # these lattices: 3 candidates x 35 steps, which also warm them up
    t0 = time.perf_counter()
    tuner = tl.Autotuner(steps=30, warmup=5)
    V, _, rows = tuner.batch_shape(f"sc-batch/{storage}", lambda V: solvers, storage, graphs=graphs, sc=True,
                                   tune_v=False)
    tune_s = time.perf_counter() - t0
    batch = tl.Batch(graphs=graphs, sc_rows=rows)
    for s in solvers:
        batch.add(s)
    batch.run(W)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(gpu_index) as clk:
        e0.record(st)
        batch.run(K)
        e1.record(st)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    info = batch.info()
    for s in solvers:
        s.finish()
    finite = sum(1 for c in cases if bool(torch.isfinite(c[0]._rho).all()))
    batch.close()
    del solvers, cases
    torch.cuda.empty_cache()
    mlups = nodes * K / (ms * 1e-3) / 1e6
    gbs = BYTES_PER_LU[storage] * nodes * K / (ms * 1e-3) / 1e9
    peak, _ = measured_peak()
    return {"MLUPS": round(mlups, 1), "GB_s": round(gbs, 1), "frac": round(gbs / peak, 4),
            "steps": K, "ms_per_step": round(ms / K, 4), "lattices": 64, "nodes": nodes,
            "groups": info["groups"], "tiles": info["tiles"], "graphs": graphs,
            "setup_s": round(setup, 1), "finite_lattices": finite,
            "autotune": {"nodes_per_thread": V, "sc_rows": rows, "seconds": round(tune_s, 1),
                         "sample": "the same 64 lattices (their first 105 steps)",
                         "trials": [{"cand": c, "ms_per_step": round(ms, 4)} for _, c, ms in tuner.trials]},
            "note": "lattices at T/Tc below about 0.78 diverge within a few hundred steps; the CPU oracle "
                    "of the reference's algorithm diverges on them alike, so the count is physics",
            "clocks": clk.summary()}


def run_served(tl, n, capacity_mlups, gpu_index, storage="fp16s", sample_alone=8, shape=None, slice_steps=200):
    """Served request stream: n seeded cylinder-channel requests (sizes
    128..2048 x NX/4, Re 20..200, log-uniform 2k..50k steps, BGK/TRT/MRT, 20%
    power law) arriving as a Poisson process at 80% of the capacity implied by
    `capacity_mlups`, served by one Server (HBM-budget admission, continuous
    batching, CUDA graphs).  Beside it: the first `sample_alone` requests run
    alone, one after another, on the plain single-lattice fp32 path."""
    import numpy as np
    import torch
    from taichi_lbm.serving import request_stream, summarize
    probe = request_stream(n, 1.0, storage=storage)
    mean_work = sum(r.nodes * r.steps for r in probe) / n
    rate = 0.8 * capacity_mlups * 1e6 / mean_work
    reqs = request_stream(n, rate, storage=storage)
    # autotune (before the stream starts) in the batch itself, on the first 32
    # requests: the members' nodes per thread and the solo threshold (a
    # lattice's fastest V alone is not its fastest in a packed mix)
    t0 = time.perf_counter()
    tuner = tl.Autotuner(steps=30, warmup=5)
    if shape:  # given, not tuned
        V, solo, form = (int(v) for v in shape.split(","))
        tuner.table["served"] = {"V": V, "solo_nodes": solo, "sc_rows": 0, "lean_form": form, "given": True}
    else:
        tuner.batch_shape("served", lambda V: [r.build(tl, nodes_per_thread=V) for r in reqs[:32]], storage)
    tune_s = time.perf_counter() - t0
    torch.cuda.empty_cache()
    srv = tl.Server(tl, hbm_budget=64 << 30, graphs=True, slice_steps=slice_steps, builders=4, autotuner=tuner)
    for r in reqs:
        srv.submit(r)
    with Clocks(gpu_index) as clk:
        done = srv.run()
    makespan = max(r.finished for r in done)
    out = summarize(done, makespan, srv.lattice_updates)
    srv.close()
    torch.cuda.empty_cache()
    # the plain fp32 drop-in, one request at a time
    alone_lu, alone_s = 0, 0.0
    for r in request_stream(sample_alone, rate, storage="fp32")[:sample_alone]:
        s = r.build(tl)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.step(r.steps, forces=True)
        torch.cuda.synchronize()
        alone_s += time.perf_counter() - t0
        alone_lu += r.steps * s.coll.group.n
        del s
    torch.cuda.empty_cache()
    out.update({"storage": storage, "rate_per_s": round(rate, 2), "mean_request_lu": round(mean_work),
                "alone_fp32_MLUPS": round(alone_lu / alone_s / 1e6, 1),
                "alone_sample": f"first {sample_alone} requests of the same stream, fp32, FusedSolver.step with "
                                "drag/lift, one after another",
                "clocks": clk.summary(),
                "autotune": {"seconds": round(tune_s, 1), "table": tuner.table,
                             "what": "nodes per thread and solo threshold of the batch, tuned on the first 32 "
                                     "requests, each candidate timed with CUDA events over 30 batched steps"}})
    out["vs_alone_fp32"] = round(out["MLUPS"] / out["alone_fp32_MLUPS"], 3)
    return out


def cpu_baseline(cfg, model, seconds):
    """The oracle (unfused reference order, OpenMP over all host cores) on
    the same lattice for about `seconds` of work."""
    from oracle import oracle as O
    from oracle.workloads import cylinder_channel_case
    meta, arrays = cylinder_channel_case(cfg["nx"], cfg["ny"], cfg["radius"], cfg["cx"], cfg["cy"],
                                         cfg["tau"], cfg["umax"], model=model,
                                         mrt_s=MRT_S if model == "mrt" else None)
    run = O.prepare(meta, arrays)
    run.step(1)  # warm-up (first touch of every page)
    n, t0 = 0, time.perf_counter()
    while True:
        run.step(1)
        n += 1
        dt = time.perf_counter() - t0
        if dt >= seconds:
            break
    run.o.close()
    active = arrays["g_fluid"].shape[0]
    return {"value": active * n / dt / 1e6, "unit": METRIC, "cores": os.cpu_count(), "kind": "port",
            "sample": f"{n} steps of the full {cfg['nx']}x{cfg['ny']} lattice ({active} updated nodes) "
                      f"in {dt:.1f} s; CPU restatement of the reference's unfused kernels, "
                      "OpenMP over all host cores (Taichi cannot be installed here)"}


def run_ours(a):
    import numpy as np  # noqa: F401
    import torch
    import taichi_lbm as tl
    rank, ws, local, dist = dist_setup()
    cfg = workload_config(a)
    K, W = a.steps, max(3, a.warmup)
    peak, peak_kind = measured_peak()
    lb, me, coll, be, solver = build(tl, cfg, a.model, a.storage, a.nodes_per_thread, a.pipeline,
                                     in_place=a.in_place)
    active = coll.group.n
    ms, clocks = time_resident(solver, K, W, dist, local)
    ms = max_over_ranks(ms, dist)
    mlups = active * K * ws / (ms * 1e-3) / 1e6
    launch_ms = ms / K
    achieved = BYTES_PER_LU[a.storage] * active / (launch_ms * 1e-3) / 1e9
    traffic = profile_traffic(a.model, a.storage)
    e2e_dt, h2d, d2h = time_e2e(lb, coll, solver, K, dist)
    e2e_dt = max_over_ranks(e2e_dt, dist)
    line = {
        "metric": METRIC, "value": round(mlups, 1), "unit": METRIC, "n_gpus": ws, "steps": K,
        "warmup": W, "ms_per_step": round(ms / K, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if a.storage == "fp32" else f"f32 compute, {a.storage} storage",
        "data": "synthetic (cylinder channel, rho=1, u=0 start)",
        "config": arm_config(a, cfg, active, solver.V, ws),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "algorithmic_bytes_per_launch": BYTES_PER_LU[a.storage] * active,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "kernel": ("one in-place step: k_aa_sites (boundary read sites), then k_aa_bulk (every "
                                "segment, phases A and B alternating) + k_aa_lanes (marked lanes, side stream), "
                                "timed together" if a.in_place else
                                "one fused step: k_fused_bulk (every segment, marked lanes skipped) + k_fused_lanes "
                                "(marked lanes, side stream), timed together"
                                if solver.launches_per_step == 2 else "one fused step (one launch)")},
        "clocks": clocks,
        "e2e": {"value": round(active * K * ws / e2e_dt / 1e6, 1), "unit": METRIC,
                "h2d_bytes_per_step": round(h2d / K, 1), "d2h_bytes_per_step": round(d2h / K, 1),
                "seconds": round(e2e_dt, 4),
                "what": "upload rho/u from pinned host memory, init_LBM, FusedSolver.step(K), "
                        "download rho/u (the inputs and result are per run; bytes are per step)"},
        "gpu_launches": K * solver.launches_per_step,
    }
    del solver, lb, me, coll, be
    torch.cuda.empty_cache()
    if not a.no_extras and ws == 1:
        extras = {}
        for model, storage, aa in (("trt", "fp32", False), ("mrt", "fp32", False), ("bgk", "fp16s", False),
                                   ("bgk", "bf16s", False), ("bgk", "i16s", False), ("bgk", "fp32", True),
                                   ("bgk", "fp16s", True)):
            if (model, storage, aa) == (a.model, a.storage, a.in_place) or (aa and a.pipeline != "direct"):
                continue
            lb2, _, coll2, _, s2 = build(tl, cfg, model, storage, None, a.pipeline, in_place=aa)
            k2 = max(10, K // 4)
            ms2, _ = time_resident(s2, k2, W, None, local)
            act = coll2.group.n
            gbs = BYTES_PER_LU[storage] * act / (ms2 / k2 * 1e-3) / 1e9
            extras[f"{model}_{storage}" + ("_in_place" if aa else "")] = {
                                            "MLUPS": round(act * k2 / (ms2 * 1e-3) / 1e6, 1),
                                            "GB_s": round(gbs, 1), "frac": round(gbs / peak, 4),
                                            "steps": k2}
            del s2, lb2, coll2
            torch.cuda.empty_cache()
        line["models"] = extras
    if not a.no_batched and ws == 1:
        kb = max(20, K // 4)
        line["batched"] = {
            "workload": "64 periodic single-component Shan-Chen lattices, side L drawn from {128, 192, ..., "
                        "1024} (seed 20261203), Carnahan-Starling a=1 b=4 R=1, G=-1, T/Tc ~ U[0.7, 0.9], "
                        "rho0 = 0.25 (1 +- 1%), BGK tau=1, Guo forcing; one persistent launch per step "
                        "over a packed tile table, CUDA graph replay",
            "bytes_per_lu": {"fp32": 72, "fp16s": 36},
            "fp32": run_batched(tl, "fp32", kb, W, local),
            "fp16s": run_batched(tl, "fp16s", kb, W, local)}
    if not a.no_served and ws == 1:
        cap = a.served_capacity or line.get("models", {}).get("bgk_fp16s", {}).get("MLUPS", 100000.0)
        line["served"] = dict(
            {"workload": f"{a.requests} cylinder-channel requests (seed 20261203): NX in {{128, 160, ..., "
                         "2048}, NY = NX/4, r = NY/10 at x = NX/5, Re ~ U[20, 200] via tau (u_max 0.04), "
                         "steps log-uniform in [2000, 50000], BGK/TRT/MRT uniform, 20% power law n ~ "
                         f"U[0.5, 1.5]; Poisson arrivals at 80% of a capacity of {cap:.0f} MLUPS; "
                         f"{a.served_storage} storage, HBM budget 64 GiB, {a.served_slice}-step slices, "
                         "CUDA graphs; diverged requests are evicted and their updates not counted"},
            **run_served(tl, a.requests, cap, local, storage=a.served_storage, sample_alone=a.alone_sample,
                         shape=a.served_shape, slice_steps=a.served_slice))
    if rank == 0 and ws == 1 and not a.no_cpu:
        line["cpu_baseline"] = cpu_baseline(cfg, a.model, a.cpu_seconds)
    if dist is not None:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- reference arm
def run_reference(a):
    """The reference path on the host cores: taichi-lbm's own Taichi code
    cannot be installed here (no package, no network), so its C++
    restatement (oracle/, same unfused kernels in the reference's call order)
    runs instead, OpenMP over every host core.  Each step is one time step of
    a band of the same channel, sized from a calibration step so the whole
    run stays within a few minutes."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    from oracle.workloads import cylinder_channel_case
    cfg = workload_config(a)
    K, W = a.steps, max(3, a.warmup)
    budget_s = 150.0

    def case(ny):
        c = dict(cfg, ny=ny, cy=ny / 2.0 - 0.5, radius=min(cfg["radius"], ny / 4.0))
        return cylinder_channel_case(c["nx"], c["ny"], c["radius"], c["cx"], c["cy"], c["tau"],
                                     c["umax"], model=a.model,
                                     mrt_s=MRT_S if a.model == "mrt" else None)

    # calibrate on a 256-row band, then size the band for the budget
    meta, arrays = case(256)
    run = O.prepare(meta, arrays)
    run.step(1)
    t0 = time.perf_counter()
    run.step(2)
    per_node = (time.perf_counter() - t0) / 2 / (cfg["nx"] * 256)
    run.o.close()
    ny = int(budget_s / max(K + W, 1) / per_node / cfg["nx"])
    ny = max(64, min(cfg["ny"], ny // 32 * 32))
    meta, arrays = case(ny)
    run = O.prepare(meta, arrays)
    run.step(W)
    t0 = time.perf_counter()
    run.step(K)
    dt = time.perf_counter() - t0
    run.o.close()
    active = arrays["g_fluid"].shape[0]
    mlups = active * K / dt / 1e6
    sample = (f"{K} steps of a {cfg['nx']}x{ny} band of the channel ({active} updated nodes per "
              "step); C++ restatement of the reference's unfused kernels (Taichi unavailable), "
              "OpenMP over all host cores")
    line = {"impl": "reference", "metric": METRIC, "value": round(mlups, 2), "unit": METRIC,
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": K, "warmup": W,
            "ms_per_step": round(dt / K * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (cylinder channel, rho=1, u=0 start)",
            "config": arm_config(a, cfg, channel_active_nodes(cfg),
                                 a.nodes_per_thread or 4,  # FusedSolver's default node width
                                 int(os.environ.get("WORLD_SIZE", "1"))),
            "cpu_baseline": {"value": round(mlups, 2), "unit": METRIC, "cores": os.cpu_count(),
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(mlups, 2), "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_mix(a):
    """The batched step of a served mix on its own: the first N requests of
    the seeded served stream (storage --mix-storage), all in the packed tile table, direct
    launches (no graph), K timed steps after W warm-up steps."""
    import torch
    import taichi_lbm as tl
    from taichi_lbm.serving import request_stream
    reqs = request_stream(a.mix_only, 20.0, storage=a.mix_storage)
    solvers = [r.build(tl, nodes_per_thread=a.mix_v) for r in reqs]
    nodes = sum(s.coll.group.n for s in solvers)
    batch = tl.Batch(graphs=a.mix_graphs, solo_nodes=a.mix_solo, lean_form=a.mix_form)
    for s in solvers:
        batch.add(s)
    batch.run(a.warmup)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    batch.run(a.steps)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.steps
    print(json.dumps({"metric": METRIC, "value": round(nodes / ms / 1e3, 1), "unit": METRIC, "steps": a.steps,
                      "warmup": a.warmup, "ms_per_step": round(ms, 4), "nodes": nodes, "info": batch.info(),
                      "config": {"workload": f"batched step of the first {a.mix_only} served requests (seed "
                                             f"20261203), {a.mix_storage}, "
                                             + (f"members of at least {a.mix_solo} nodes solo" if a.mix_solo
                                                else "every member packed")
                                             + (", CUDA graphs" if a.mix_graphs else ", direct launches"),
                                 "nodes_per_thread": solvers[0].V, "lean_form": a.mix_form}}))
    batch.close()


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.batched_only:
        import taichi_lbm as tl
        print(json.dumps({"batched": run_batched(tl, a.batched_only, a.steps, max(3, a.warmup), 0)}))
    elif a.mix_only:
        run_mix(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
