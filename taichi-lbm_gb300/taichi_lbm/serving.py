"""Serving: simulations admitted as they arrive, run together, returned as
they finish.

A Server keeps one Batch.  Each request is a cylinder-channel simulation
(lattice size, collision model, relaxation time or power-law fluid, step
count) whose populations, mask-derived plan and boundary groups stay on the
device from admission to completion.  Admission is against an HBM budget:
a request waits in FIFO order until the bytes its lattice needs fit beside
the running ones.  The loop is continuous batching: it advances every
member by a slice of steps (at most `slice_steps`, never past the member
that finishes first), retires finished members, and admits the requests
that arrived meanwhile, so work arriving while others run shares the GPU
with them.  A request's lattice is built by a builder thread on its own
stream while the batch runs, and joins the batch at the next slice
boundary after it is ready.

Each result is the same as running the request alone (FusedSolver.step with
forces), because a batch computes every member with the single-lattice
arithmetic (see Batch).  Latency is completion minus arrival, in seconds of
the server's clock.

Failure detection: every member plan has a device status word that its
kernels set when a colliding node's populations turn NaN or infinite, when
the fixed-point storage saturates, or when its drag/lift monitor sums to a
non-finite force.  After each slice the members' words are copied to pinned
host memory behind the slice's event; once that event has completed, a
member with a bit set leaves the batch at the next slice boundary without
touching the others.  A fixed-point member that only saturated (its flow
left the storage's range, typically in the pressure transient of the
impulsive start) is built again with a step twice as coarse (range twice as
wide, down to fixed_exp 17) and queued ahead of new arrivals; its latency
counts from its first arrival.  A member that turned non-finite, or still
saturates at the coarsest step, is evicted (retired with ``failed`` set).
The lattice updates of discarded attempts and of evicted requests are not
counted in the aggregate.
"""
import collections
import time
import warnings

import numpy as np
import torch

from . import _capi as A
from .batch import Batch
from .workloads import cylinder_channel


class Request:
    """One simulation: an NX x NY channel with a cylinder of radius NY/10
    at x = NX/5 (centre height NY/2), parabolic inlet u_max, model
    "bgk" | "trt" | "mrt", relaxation time tau or a power-law fluid (m, n),
    `steps` time steps, arriving at `arrival` seconds."""

    def __init__(self, rid, nx, ny, model, tau, steps, arrival=0.0, powerlaw=None, umax=0.04,
                 storage="fp16s", fixed_exp=None):
        self.rid, self.nx, self.ny = rid, int(nx), int(ny)
        self.model, self.tau, self.steps = model, float(tau), int(steps)
        self.arrival, self.powerlaw, self.umax, self.storage = float(arrival), powerlaw, umax, storage
        self.admitted = self.finished = None
        self.forces = None      # (steps, 2) float64 numpy: drag, lift per step
        self.fields = None      # optional final fields (keep_fields)
        self.finite = None
        self.updated_nodes = None
        self.updates = 0        # lattice updates run for this request
        self.failed = None      # status bits that evicted it (diverged), else None
        self.steps_run = 0
        self.fixed_exp = fixed_exp  # fixed-point step 2^-fixed_exp (None: the default)
        self.retries = 0        # rebuilds with a coarser fixed-point step
        self.retry = False

    @property
    def nodes(self):
        return self.nx * self.ny

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival

    def tune_key(self):
        """Autotuner table key of this request's shape."""
        from .autotune import Autotuner
        return Autotuner.key(self.model, self.storage, self.nodes, powerlaw=self.powerlaw is not None)

    def build(self, tl, keep_init=False, nodes_per_thread=None):
        """The request's lattice and solver (cylinder_channel + FusedSolver)."""
        r = self.ny / 10.0
        s = [0.0, 1.64, 1.54, 0.0, 1.7, 0.0, 1.7, 1.0 / self.tau, 1.0 / self.tau] if self.model == "mrt" else None
        lb, me, coll, be = cylinder_channel(tl, self.nx, self.ny, r, self.nx / 5.0, self.ny / 2.0 - 0.5, self.tau,
                                            self.umax, model=self.model, mrt_s=s, keep_init=keep_init,
                                            name=f"req{self.rid}", powerlaw=self.powerlaw)
        return tl.FusedSolver(lb, me, coll, be, storage=self.storage, nodes_per_thread=nodes_per_thread,
                              fixed_exp=self.fixed_exp)


def device_bytes(nx, ny, storage):
    """Bytes of device memory a request of this size holds while served: the
    LBField's fp32 populations and fields, the plan's population buffers
    (fp32 or 16-bit), saved moments, node codes and monitors."""
    pitch = (nx + 31) // 32 * 32
    per = (2 * 9 * 4            # LBField f, f2 (fp32)
           + 12 * 4             # rho, total_rho, vel, force, pressure, ... (fp32 fields)
           + 9 * 4              # collision state (tau / MRT diag)
           + 2 * 3 * 4          # plan moments (two parities)
           + 2 + 1)             # node code, mask
    if storage != "fp32":
        per += 2 * 9 * 2        # 16-bit population buffers
    return per * pitch * ny + (1 << 20)


class Server:
    """builders: host threads that build arriving requests' lattices (each
    on its own CUDA stream) while the scheduler keeps the GPU busy."""

    def __init__(self, tl, hbm_budget, graphs=True, slice_steps=200, keep_fields=False, builders=1, ahead=2,
                 reserve_bytes=16 << 30, autotuner=None, batch_key="served"):
        """autotuner: an Autotuner whose table gives the batch's shape (entry
        `batch_key`: solo threshold and, when tuned in the batch, the nodes per
        thread of every member) or else each request's nodes per thread (by
        Request.tune_key); shapes it has no entry for keep the defaults."""
        self.tl = tl
        self.autotuner = autotuner
        self.batch_key = batch_key
        self.batch = Batch(graphs=graphs, **(autotuner.batch_kwargs(batch_key) if autotuner else {}))
        self.budget = int(hbm_budget)
        self.used = 0
        self.slice_steps = int(slice_steps)
        self.keep_fields = keep_fields
        self.builders = max(1, int(builders))
        self.ahead = max(1, int(ahead))  # slices queued on the GPU before the scheduler waits
        self.reserve_bytes = int(reserve_bytes)
        self.queue = collections.deque()
        self.requeue = []       # saturated fixed-point requests to build again
        self.min_fixed_exp = 17
        self.active = {}        # slot -> [request, solver, remaining steps, bytes]
        self.done = []
        self.lattice_updates = 0

    def submit(self, req):
        if device_bytes(req.nx, req.ny, req.storage) > self.budget:
            raise ValueError(f"request {req.rid} needs more than the whole HBM budget")
        self.queue.append(req)

    def _build(self, req, stream):
        """Builder thread: lattice, plan, first step and first drag/lift row
        on `stream`; returns what the scheduler needs to join the batch."""
        V = None
        if self.autotuner:
            V = self.autotuner.table.get(self.batch_key, {}).get("V")
            if V is None:
                V = self.autotuner.lookup(req.tune_key(), "V")
        with torch.cuda.stream(stream):
            solver = req.build(self.tl, nodes_per_thread=V)
            mon = Batch.prepare(solver, req.steps)
            ev = torch.cuda.Event()
            ev.record(stream)
        return solver, mon, ev

    def _join(self, req, built, now):
        solver, mon, ev = built
        torch.cuda.current_stream().wait_event(ev)
        slot = self.batch.add(solver, req.steps, prepared=mon)
        req.admitted = now
        req.updated_nodes = int(solver.coll.group.n)  # nodes a step updates (fluid and boundary)
        self.active[slot] = [req, solver, req.steps - 1, device_bytes(req.nx, req.ny, req.storage)]

    def _retire(self, entry, now_fn):
        """Finish a member that left the batch: on the retire stream, after
        the event of the slice it finished in (later slices keep running).
        A member marked for a retry is dropped and queued again instead."""
        (req, solver, _, nbytes), mon, ev = entry
        if req.retry:
            with torch.cuda.stream(self.retire_stream):
                self.retire_stream.wait_event(ev)
                solver.status.zero_()
                self.retire_stream.synchronize()
            req.retry = False
            req.retries += 1
            req.fixed_exp = (req.fixed_exp or A.FIXED_EXP_DEFAULT) - 1
            req.updates = req.steps_run = 0
            self.used -= nbytes
            self.requeue.append(req)
            return
        with torch.cuda.stream(self.retire_stream):
            self.retire_stream.wait_event(ev)
            _, series, count = mon
            n = min(int(count.item()), series.shape[0])
            req.forces = series[:n].cpu().numpy()
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")  # a diverged member's finish() warns; its status says so
                solver.finish()
            if req.failed is None and solver.status_bits:
                req.failed = solver.status_bits
            req.finite = bool(torch.isfinite(solver.lb._rho).all()) and req.failed is None
            if self.keep_fields:
                req.fields = {"rho": solver.lb.rho.to_numpy(), "vel": solver.lb.vel.to_numpy()}
            self.retire_stream.synchronize()
        req.finished = now_fn()
        self.used -= nbytes
        self.done.append(req)

    def _check(self, slots, host):
        """Status words of a completed slice (pinned host copy): members
        with a bit set are marked to leave, for a retry with a coarser
        fixed-point step (saturation alone) or for eviction."""
        for slot, bits in zip(slots, host.tolist()):
            a = self.active.get(slot)
            if not bits or a is None or a[0].failed is not None or a[0].retry:
                continue
            req = a[0]
            e = req.fixed_exp or A.FIXED_EXP_DEFAULT
            if (bits == A.STATUS_SATURATED and req.storage == "i16s" and e > self.min_fixed_exp):
                req.retry = True
            else:
                req.failed = int(bits)
            a[2] = 0  # leaves at the next slice boundary

    def _leave(self, retiring):
        """Members at zero remaining steps leave the batch (no wait); their
        retirement is queued behind an event of the current stream."""
        gone = [s for s, a in self.active.items() if a[2] <= 0]
        if not gone:
            return
        ev = torch.cuda.Event()
        ev.record()
        for slot in gone:
            mon = self.batch.members[slot][1]
            self.batch.remove(slot)
            retiring.append((self.active.pop(slot), mon, ev))

    def run(self, clock=time.perf_counter):
        """Serve every submitted request (arrival times relative to the start
        of run); returns the finished requests in completion order."""
        import concurrent.futures as cf
        t0 = clock()

        def now():
            return clock() - t0

        pending = collections.deque(sorted(self.queue, key=lambda r: r.arrival))
        self.queue.clear()
        # builders' and retirement's short kernels go ahead of the batch's
        # persistent ones: high stream priority
        hi = torch.cuda.Stream.priority_range()[1] if hasattr(torch.cuda.Stream, "priority_range") else -1
        streams = [torch.cuda.Stream(priority=hi) for _ in range(self.builders)]
        self.retire_stream = torch.cuda.Stream(priority=hi)
        # lattices of every size come and go: give each builder stream one
        # large cached segment up front, so building carves tensors out of it
        # instead of calling the driver allocator per tensor
        reserve = min(self.budget, self.reserve_bytes) // self.builders
        for st in streams:
            with torch.cuda.stream(st):
                del_me = torch.empty(reserve, dtype=torch.uint8, device="cuda")
                del del_me
        building = collections.deque()  # (request, future) in admission order
        retiring = []                   # members that left, with the event to wait for
        inflight = collections.deque()  # end events of the slices queued on the GPU
        # the scheduler's own stream: nothing implicit (work on the legacy
        # default stream from any thread) queues behind the batch's slices
        sched = torch.cuda.Stream()
        with cf.ThreadPoolExecutor(self.builders) as pool, torch.cuda.stream(sched):
            n_started = 0
            while pending or building or self.active or retiring or self.requeue:
                t = now()
                while self.requeue:  # retries go ahead of new arrivals
                    pending.appendleft(self.requeue.pop())
                # admission: arrived requests whose lattice fits the budget go to a builder
                while pending and pending[0].arrival <= t and \
                        self.used + device_bytes(pending[0].nx, pending[0].ny, pending[0].storage) <= self.budget:
                    req = pending.popleft()
                    self.used += device_bytes(req.nx, req.ny, req.storage)
                    building.append((req, pool.submit(self._build, req, streams[n_started % self.builders])))
                    n_started += 1
                # built lattices join the batch in admission order
                while building and building[0][1].done():
                    req, fut = building.popleft()
                    self._join(req, fut.result(), now())
                self._leave(retiring)  # single-step requests
                launched = False
                if self.active:
                    # at most `ahead` slices queued: the scheduler (and the
                    # builders' small GPU steps) stay close to the GPU's clock
                    while len(inflight) >= self.ahead:
                        ev0, slots0, host0 = inflight.popleft()
                        ev0.synchronize()
                        self._check(slots0, host0)
                    self._leave(retiring)  # evicted members leave before the next slice
                if self.active:
                    k = min(self.slice_steps, min(a[2] for a in self.active.values()))
                    self.batch.run(k)
                    # the members' status words, copied behind the slice
                    slots = list(self.active)
                    host = torch.empty(len(slots), dtype=torch.int32, pin_memory=True)
                    host.copy_(torch.stack([self.active[sl][1].status[0] for sl in slots]), non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record()
                    inflight.append((ev, slots, host))
                    launched = True
                    for a in self.active.values():
                        a[2] -= k
                        a[0].updates += k * a[0].updated_nodes
                        a[0].steps_run += k
                # retire what finished in earlier slices while this one runs
                for entry in retiring:
                    self._retire(entry, now)
                retiring = []
                if launched:
                    self._leave(retiring)
                elif building:
                    building[0][1].result()
                elif pending:
                    time.sleep(max(0.0, min(pending[0].arrival - now(), 0.001)))
        for ev0, slots0, host0 in inflight:
            ev0.synchronize()
        for r in self.done:
            r.updates += r.updated_nodes  # the staged first step of each request
            if r.failed is None:  # evicted (diverged) requests' work is not counted
                self.lattice_updates += r.updates
        return self.done

    def close(self):
        self.batch.close()


def request_stream(n, rate, seed=20261203, nx_choices=tuple(range(128, 2049, 32)), steps=(2000, 50000),
                   re_range=(20.0, 200.0), umax=0.04, powerlaw_fraction=0.2, n_range=(0.5, 1.5),
                   storage="fp16s"):
    """Seeded cylinder-channel requests with Poisson arrivals at `rate` per
    second: NX uniform over nx_choices, NY = NX/4, cylinder radius NY/10,
    Re ~ U[re_range] through tau = 0.5 + 3 u_max (2r) / Re, steps log-uniform
    in `steps`, model uniform over BGK/TRT/MRT, a fraction of power-law
    fluids with n ~ U[n_range] and consistency m giving the same Re,
    m = u_max^(2-n) (2r)^n / Re."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        nx = int(rng.choice(np.asarray(nx_choices)))
        ny = nx // 4
        d = 2.0 * ny / 10.0
        re = rng.uniform(*re_range)
        tau = 0.5 + 3.0 * umax * d / re
        st = int(round(np.exp(rng.uniform(np.log(steps[0]), np.log(steps[1])))))
        model = ["bgk", "trt", "mrt"][int(rng.integers(3))]
        pl = None
        if rng.uniform() < powerlaw_fraction:
            nn = rng.uniform(*n_range)
            pl = (umax ** (2.0 - nn) * d ** nn / re, nn)
        out.append(Request(i, nx, ny, model, tau, st, arrival=t, powerlaw=pl, umax=umax, storage=storage))
    return out


def summarize(done, makespan, lattice_updates):
    lat = np.array([r.latency for r in done])
    return {"requests": len(done), "makespan_s": round(makespan, 3),
            "MLUPS": round(lattice_updates / makespan / 1e6, 1),
            "p50_s": round(float(np.percentile(lat, 50)), 4), "p99_s": round(float(np.percentile(lat, 99)), 4),
            "finite": int(sum(1 for r in done if r.finite)),
            "nonfinite_requests": sorted(int(r.rid) for r in done if not r.finite),
            "evicted_requests": sorted(int(r.rid) for r in done if r.failed is not None)}
