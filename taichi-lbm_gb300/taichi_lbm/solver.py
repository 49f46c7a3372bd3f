"""FusedSolver: the whole reference step as one CUDA kernel per time step.

The reference leaves the step composition to the user's ``lbm_solve()``
(cases/Circular cylinder.py:182-193, cases/Power Law Fluid.py:160-173):

    density -> pressure -> force_density -> velocity
    [-> shear_rate -> relaxation_time]   (power-law fluid)
    -> collision.apply -> boundary_engine.apply_boundary_conditions

``FusedSolver(lb_field, macroscopic_engine, collision, boundary_engine)``
runs exactly that composition; ``step(n)`` equals n calls of that
``lbm_solve()`` followed by the moment prologue of the next step (so ``rho``
and ``vel`` hold the moments of the final ``f``).  Internally: the first
collision runs through the per-stage kernels, then n-1 fused launches (each
= boundary pass of step k-1 + moments/collision of step k), then one stream
and boundary pass and the moment kernels.

``in_place=True`` runs the fused steps on one population buffer (the
AA-pattern: alternating phases whose nodes read and write the same nine
locations) instead of the ping-pong pair; the results are the same bits.
"""
import ctypes
import warnings
import zlib

import numpy as np
import torch

from . import _capi as A
from ._plan import BoundaryItem, UnsupportedComposition, compile_plan
from .boundary import BoundaryCondition
from .collision import BGKCollision, MRTCollision, PowerLawFluid, TRTCollision
from .lbm import stream_handle

# "i16s": int16 fixed point (steps of 2^-fixed_exp, default 2^-19) of
# f - w_k rho_ref; every collision conserves each node's stored mass exactly
STORAGE = {"fp32": A.STORE_F32, "fp16s": A.STORE_F16S, "bf16s": A.STORE_BF16S, "i16s": A.STORE_I16S}
DEFAULT_V = {A.STORE_F32: 4, A.STORE_F16S: 4, A.STORE_BF16S: 4, A.STORE_I16S: 4}
STATE_DTYPE = {A.STORE_F16S: torch.float16, A.STORE_BF16S: torch.bfloat16, A.STORE_I16S: torch.int16}
PIPELINE = {"direct": A.PIPE_DIRECT, "async": A.PIPE_ASYNC, "prefetch": A.PIPE_PREFETCH}


def boundary_items(boundary_engine):
    items = []
    for name, bc in boundary_engine.boundary_conditions.items():
        if not isinstance(bc, BoundaryCondition):
            raise UnsupportedComposition(f"boundary '{name}' is not a BoundaryCondition")
        vel = None
        if hasattr(bc, "velocity_value"):
            vel = bc.per_node_velocity_host()
        items.append(BoundaryItem(bc.kind, bc.group.nodes, getattr(bc, "direction", 0),
                                  getattr(bc, "rho_value", 0.0), vel, name))
    return items


class FusedSolver:
    def __init__(self, lb_field, macroscopic_engine, collision, boundary_engine, storage="fp32",
                 nodes_per_thread=None, local_relaxation=None, pipeline="direct", tune=0,
                 sc_boundary_engine=None, two_pass=True, rho_ref=None, overlap=True, lane_special=True,
                 fixed_exp=None, wait_cycles=0, in_place=False):
        if lb_field.nc > 1:
            raise UnsupportedComposition("the fused step is single-component; a multi-component lattice "
                                         "runs the per-stage kernels")
        self.sc = lb_field.sc_field
        # fixed-point storage: step 2^-fixed_exp, range |f - w rho_ref| < 2^(15 - fixed_exp)
        self.fixed_exp = int(fixed_exp) if fixed_exp is not None else A.FIXED_EXP_DEFAULT
        self.wait_cycles = int(wait_cycles)
        self.status_bits = 0
        # in-place (AA-pattern) step: one population buffer instead of two
        self.in_place = bool(in_place)
        if self.in_place and (lb_field.sc_field is not None or pipeline != "direct" or not two_pass
                              or not lane_special):
            raise UnsupportedComposition("the in-place step runs the direct two-pass pipeline with "
                                         "lane-granular special work, without Shan-Chen")
        self.lane_special = bool(lane_special)
        self.two_pass = bool(two_pass)
        self.overlap = bool(overlap)
        self.rho_ref = rho_ref
        self.bsc = sc_boundary_engine
        if self.sc is not None:
            from .shanchen import PeriodicPsi_BT, PeriodicPsi_LR, ShanChenForceC1
            if not isinstance(self.sc, ShanChenForceC1):
                raise UnsupportedComposition("the fused Shan-Chen step is single-component")
            kinds = {type(b) for b in (sc_boundary_engine.boundary_conditions.values()
                                       if sc_boundary_engine is not None else [])}
            if kinds != {PeriodicPsi_LR, PeriodicPsi_BT}:
                raise UnsupportedComposition("the fused Shan-Chen step needs the psi boundaries "
                                             "PeriodicPsi_LR and PeriodicPsi_BT (a periodic lattice)")
            if pipeline != "direct":
                raise UnsupportedComposition("the fused Shan-Chen step runs the direct pipeline")
        self.lb = lb_field
        self.me = macroscopic_engine
        self.coll = collision
        self.be = boundary_engine
        self.storage = STORAGE[storage] if isinstance(storage, str) else int(storage)
        self.pipeline = PIPELINE[pipeline] if isinstance(pipeline, str) else int(pipeline)
        self.V = int(nodes_per_thread or DEFAULT_V[self.storage])
        self.tune = int(tune)
        if self.pipeline != A.PIPE_DIRECT and not (self.pipeline == A.PIPE_PREFETCH and self.V == 8
                                                   and self.storage != A.STORE_F32 and two_pass):
            self.V = 4
        self.status = torch.zeros(1, dtype=torch.int32, device=lb_field.device)
        if local_relaxation is None:
            local_relaxation = isinstance(collision.fluid_model, PowerLawFluid)
        self.powerlaw = bool(local_relaxation)
        if self.powerlaw and not isinstance(collision.fluid_model, PowerLawFluid):
            raise UnsupportedComposition("local relaxation needs a PowerLawFluid")
        if macroscopic_engine.group is not collision.group and not np.array_equal(
                macroscopic_engine.group.nodes, collision.group.nodes):
            raise UnsupportedComposition("the macroscopic and collision groups differ")
        self.group = collision.group
        self._plan = None
        self._owns = False
        self._build()

    # ------------------------------------------------------------ build
    def _rho_ref(self):
        """Reference density of the 16-bit storage shift: the mean density of
        the collision group at plan build (1 when the lattice holds none yet)."""
        if self.rho_ref is not None:
            return float(self.rho_ref)
        nd = torch.as_tensor(self.group.nodes, device=self.lb._rho.device).long()
        if nd.numel() == 0:
            return 1.0
        r = float(self.lb._rho[nd[:, 1], nd[:, 0]].double().mean().item())
        return r if np.isfinite(r) and r > 0.0 else 1.0

    def _uniform(self, field_tensor, planes=None):
        nd = torch.as_tensor(self.group.nodes, device=field_tensor.device).long()
        if planes is None:
            v = field_tensor[nd[:, 1], nd[:, 0]]
            vals = torch.unique(v)
            if vals.numel() != 1:
                raise UnsupportedComposition("per-node relaxation times differ across the group "
                                             "(Newtonian fused path needs a uniform tau)")
            return float(vals[0].item())
        out = []
        for a in planes:
            vals = torch.unique(field_tensor[a][nd[:, 1], nd[:, 0]])
            if vals.numel() != 1:
                raise UnsupportedComposition(f"MRT rate s{a} differs across the group")
            out.append(float(vals[0].item()))
        return out

    def _build(self):
        lb, c = self.lb, self.coll
        nx, ny, P = lb.NX, lb.NY, lb.pitch
        cp = compile_plan(nx, ny, self.group.nodes, lb.links_host(), boundary_items(self.be), self.V,
                          in_place=self.in_place)
        self.compiled = cp
        dev = lb.device
        d = A.LbmPlanDesc()
        d.nx, d.ny, d.pitch = nx, ny, P
        d.storage = self.storage
        d.nodes_per_thread = self.V
        d.pipeline = self.pipeline
        d.tune = self.tune
        d.fluid_model = A.POWERLAW if self.powerlaw else A.NEWTONIAN
        d.tau_min, d.tau_max = float(c.tau_min), float(c.tau_max)
        if self.powerlaw:
            d.pl_m, d.pl_n = float(c.fluid_model.m), float(c.fluid_model.n)
        if isinstance(c, BGKCollision):
            d.model = A.BGK
            self.tau_state = c._tau
            d.tau = 1.0 if self.powerlaw else self._uniform(c._tau)
        elif isinstance(c, TRTCollision):
            d.model = A.TRT
            d.magic = float(c.magic[0])
            self.tau_state = c._tau_sym
            if not self.powerlaw:
                d.tau = self._uniform(c._tau_sym)
                d.tau_antisym = self._uniform(c._tau_antisym)
            else:
                d.tau = d.tau_antisym = 1.0
        elif isinstance(c, MRTCollision):
            d.model = A.MRT
            self.tau_state = c._diag[7]
            planes = [0, 1, 2, 3, 4, 5, 6] + ([] if self.powerlaw else [7, 8])
            s = self._uniform(c._diag, planes)
            for a, v in zip(planes, s):
                d.mrt_s[a] = v
            d.tau = 1.0
            if self.powerlaw and not torch.equal(c._diag[7], c._diag[8]):
                raise UnsupportedComposition("MRT power law needs diag[7] == diag[8]")
        else:
            raise UnsupportedComposition(f"unknown collision {type(c).__name__}")
        g = np.asarray(lb.gravity_force, np.float32).reshape(2)
        d.gravity[0], d.gravity[1] = float(g[0]), float(g[1])
        if self.sc is not None:
            if cp.instances or not (cp.code == A.CODE_ACTIVE).all():
                raise UnsupportedComposition("the fused Shan-Chen step needs every node colliding and "
                                             "streaming periodically, with no rewrite boundaries")
            if self.powerlaw:
                raise UnsupportedComposition("the fused Shan-Chen step is Newtonian")
            d.sc = 1
            d.g_coh = float(self.sc.g_coh)
            d.sc_T = self._uniform(lb._T)
            d.eos = self.sc.psi.struct()

        # device-side plan data
        self.code = torch.zeros((ny, P), dtype=torch.int16, device=dev)
        self.code[:, :nx] = torch.as_tensor(cp.code.T.astype(np.int16), device=dev)
        self.seg_flags = torch.as_tensor(cp.seg_flags, device=dev)
        self.bc_vel = None
        if cp.bc_vel is not None:
            self.bc_vel = torch.zeros((2, ny, P), dtype=torch.float32, device=dev)
            self.bc_vel[:, :, :nx] = torch.as_tensor(np.transpose(cp.bc_vel, (0, 2, 1)).copy(),
                                                     device=dev)
        d.nbc = len(cp.instances)
        for n, ins in enumerate(cp.instances):
            b = d.bc[n]
            b.kind, b.direction, b.rho_value = ins["kind"], ins["direction"], ins["rho_value"]
            b.velocity_per_node = (self.bc_vel.data_ptr()
                                   if ins["kind"] in (A.BC_VELOCITY_BB, A.BC_VELOCITY_EQ,
                                                      A.BC_VELOCITY_NEEM) else None)
        d.nprog = cp.nprog
        for p in range(A.MAX_PROG):
            for s in range(A.PROG_LEN):
                d.prog[p][s] = int(cp.programs[p, s])
        d.rho_ref = self._rho_ref()
        d.fixed_exp = self.fixed_exp
        d.wait_cycles = self.wait_cycles
        d.aa = 1 if self.in_place else 0
        self.desc = d
        # flagged segments, listed for the two-pass direct step
        flags = np.asarray(cp.seg_flags).ravel()
        flagged = np.flatnonzero(flags).astype(np.int32)
        plain = np.flatnonzero(flags == 0).astype(np.int32)
        self.special = torch.as_tensor(flagged if flagged.size else np.zeros(1, np.int32), device=dev)
        self.nspecial = int(flagged.size)
        self.plain = torch.as_tensor(plain if plain.size else np.zeros(1, np.int32), device=dev)
        self.nplain = int(plain.size)
        self.lane_mask = torch.as_tensor(cp.lane_mask.view(np.int32), device=dev)
        self.lanes = torch.as_tensor(cp.lanes if cp.lanes.size else np.zeros(1, np.int32), device=dev)
        self.nlanes = int(cp.lanes.size)
        self.mom = [torch.zeros((3, ny, P), dtype=torch.float32, device=dev) for _ in range(2)]
        if self.storage == A.STORE_F32:
            self.fbuf = None
        else:
            self.fbuf = [torch.zeros((9, ny, P), dtype=STATE_DTYPE[self.storage], device=dev)
                         for _ in range(1 if self.in_place else 2)]
        self.aa_sites = self.aa_vals = None
        if self.in_place:
            rs = cp.read_sites
            q = (rs[:, 1].astype(np.int64) * P + rs[:, 0]).astype(np.int32)
            self.aa_nsites = int(q.size)
            self.aa_sites = torch.as_tensor(q if q.size else np.zeros(1, np.int32), device=dev)
            self.aa_vals = torch.zeros(max(q.size, 1) * 9, dtype=torch.float32, device=dev)
        plan = ctypes.c_void_p()
        A.call("lbm_plan_create", ctypes.byref(d), ctypes.byref(plan))
        self._plan = plan
        self.parity = 0

    def __del__(self):
        try:
            if self._plan is not None:
                A.load().lbm_plan_destroy(self._plan)
        except Exception:
            pass

    # ------------------------------------------------------------ running
    def _bind(self):
        lb = self.lb
        b = A.LbmPlanBuffers()
        bufs = self._state_buffers()
        b.fa, b.fb = bufs[0].data_ptr(), bufs[-1].data_ptr()  # in place: one buffer, fa == fb
        if self.in_place:
            b.aa_sites, b.aa_nsites, b.aa_vals = (self.aa_sites.data_ptr(), self.aa_nsites,
                                                  self.aa_vals.data_ptr())
        b.mom_a, b.mom_b = self.mom[0].data_ptr(), self.mom[1].data_ptr()
        b.code = self.code.data_ptr()
        b.seg_flags = self.seg_flags.data_ptr()
        b.bc_vel = None if self.bc_vel is None else self.bc_vel.data_ptr()
        b.tau = self.tau_state.data_ptr() if self.powerlaw else None
        b.status = self.status.data_ptr()
        if self.two_pass and self.pipeline in (A.PIPE_DIRECT, A.PIPE_PREFETCH):
            b.special, b.nspecial = self.special.data_ptr(), self.nspecial
            b.special_stream = 1 if self.overlap else 0
            if self.pipeline == A.PIPE_PREFETCH:
                b.plain, b.nplain = self.plain.data_ptr(), self.nplain
            elif self.lane_special:
                b.lane_mask, b.lanes, b.nlanes = self.lane_mask.data_ptr(), self.lanes.data_ptr(), self.nlanes
        A.call("lbm_plan_bind", self._plan, ctypes.byref(b))

    def _moments(self):
        """The moment stages of a step (with the Shan-Chen force when present)."""
        lb, me = self.lb, self.me
        me.density(lb)
        me.pressure(lb)
        if self.sc is not None:
            self.sc.update_psi(lb)
            self.bsc.apply_boundary_conditions(lb)
            self.sc.cau_SCforce(lb)
        me.force_density(lb)
        me.velocity(lb)

    def _staged_first_step(self):
        lb, c = self.lb, self.coll
        self._moments()
        if self.powerlaw:
            c.shear_rate(lb)
            c.relaxation_time(lb)
        c.apply(lb)

    def begin(self):
        """Run the first collision and load the fused state (f2, moments)."""
        lb = self.lb
        self._staged_first_step()
        self._bind()
        A.call("lbm_plan_set_parity", self._plan, 0)
        self.mom[0][0].copy_(lb._rho)
        self.mom[0][1:3].copy_(lb._vel)
        if self.fbuf is not None:  # both buffers (a step never writes nodes outside the group)
            A.call("lbm_plan_import", self._plan, ctypes.c_void_p(lb._f2.data_ptr()), stream_handle())
        elif not self.in_place:  # fp32: f2 is the state, f the other buffer; make them agree
            lb._f.copy_(lb._f2)
        lb._fused_owner = self
        self._live = True

    @property
    def launches_per_step(self):
        """Kernel launches of one lbm_plan_run step: two for the two-pass
        direct step (plain segments, then the listed ones), else one."""
        if self.in_place:  # the boundary read sites, the marked lanes, the plain segments
            return (1 if self.aa_nsites else 0) + (1 if self.nlanes else 0) + 1
        if (self.sc is None and self.pipeline in (A.PIPE_DIRECT, A.PIPE_PREFETCH) and self.two_pass
                and self.nspecial and (self.nplain or self.pipeline == A.PIPE_DIRECT)):
            return 2
        return 1

    def run(self, nsteps):
        """nsteps fused steps on the current state (no staging)."""
        A.call("lbm_plan_run", self._plan, int(nsteps), stream_handle())

    @property
    def saturated(self):
        """The fixed-point storage clamped a colliding node's value (or met a
        non-finite one) during the last run: set from the device status word
        at finish()."""
        return bool(self.status_bits & A.STATUS_SATURATED)

    @property
    def nonfinite(self):
        """A colliding node's post-collision value was NaN or infinite during
        the last run (floating-point storages), read at finish()."""
        return bool(self.status_bits & A.STATUS_NONFINITE)

    def read_status(self):
        """The device status word's sticky LBM_STATUS_* bits of the current run
        (synchronises with the current stream)."""
        return int(self.status.item())

    def finish(self):
        """Last stream/boundary pass and moment prologue; f, f2, rho, vel current."""
        lb = self.lb
        lb._fused_owner = None
        self._live = False
        self.status_bits = self.read_status()
        self.status.zero_()
        if self.status_bits & A.STATUS_TIMEOUT:
            raise A.LbmError("fused step: a wait on a shared-memory copy exceeded its time budget; "
                             "the state is invalid")
        par = ctypes.c_int32()
        A.call("lbm_plan_get_parity", self._plan, ctypes.byref(par))
        s = stream_handle()
        if self.nonfinite:
            warnings.warn("fused run: a colliding node's populations became NaN or infinite (the flow "
                          "diverged)")
        if self.fbuf is None:
            if par.value == 0 or self.in_place:  # state in f2 -> write f
                A.call("lbm_plan_stream", self._plan, ctypes.c_void_p(lb._f.data_ptr()), s)
            else:  # state in f's storage -> stream into f2's storage, then swap roles
                A.call("lbm_plan_stream", self._plan, ctypes.c_void_p(lb._f2.data_ptr()), s)
                lb._f, lb._f2 = lb._f2, lb._f
        else:
            if self.storage == A.STORE_I16S and self.saturated:
                rng = 2.0 ** (15 - self.fixed_exp)
                warnings.warn(f"fixed-point storage saturated: a colliding node left |f - w rho_ref| < "
                              f"{rng:g} (fixed_exp={self.fixed_exp}); use a smaller fixed_exp, or fp32 or "
                              "fp16s, for this flow")
            A.call("lbm_plan_stream", self._plan, ctypes.c_void_p(lb._f.data_ptr()), s)
            A.call("lbm_plan_export", self._plan, ctypes.c_void_p(lb._f2.data_ptr()), s)
        if self.powerlaw:
            c = self.coll
            nd = torch.as_tensor(self.group.nodes, device=lb.device).long()
            if isinstance(c, TRTCollision):
                ts = c._tau_sym[nd[:, 1], nd[:, 0]]
                c._tau_antisym[nd[:, 1], nd[:, 0]] = float(c.magic[0]) / (ts - 0.5) + 0.5
            elif isinstance(c, MRTCollision):
                c._diag[8].copy_(c._diag[7])
        self._moments()

    def sync(self):
        if getattr(self, "_live", False):
            self.finish()

    # ------------------------------------------------------------ checkpoint / resume
    CHECKPOINT_FORMAT = "taichi_lbm.fused.v1"

    def _fingerprint(self):
        """What a checkpoint must match: lattice shape, storage, model and the
        compiled node codes (geometry and boundary programs)."""
        d = self.desc
        return {"nx": int(d.nx), "ny": int(d.ny), "pitch": int(d.pitch), "storage": int(self.storage),
                "model": int(d.model), "fluid_model": int(d.fluid_model), "sc": int(d.sc), "aa": int(d.aa),
                "code_crc": zlib.crc32(np.ascontiguousarray(self.compiled.code).tobytes())}

    def _state_buffers(self):
        # the ping-pong buffers in bind order (fa, fb), or the in-place one
        if self.fbuf is not None:
            return list(self.fbuf)
        return [self.lb._f2] if self.in_place else [self.lb._f2, self.lb._f]

    def checkpoint(self):
        """Snapshot of a live run (between begin() and finish()) as CPU tensors:
        both population buffers in their storage type (the 16-bit shifted
        values as stored, so nothing is rounded twice), both saved-moment
        buffers, the per-node relaxation state of a power-law run, the
        ping-pong parity and LBField.time.  torch.save() writes it to disk;
        restore() on a solver built for the same lattice resumes from it, and
        the resumed run equals the uninterrupted one to the bit.  Queued work
        on the current stream finishes first (the copies are ordered after it)."""
        if not getattr(self, "_live", False):
            raise RuntimeError("checkpoint() needs a live run (between begin() and finish())")
        ck = {"format": self.CHECKPOINT_FORMAT, "plan": self._fingerprint(), "parity": self.parity_now(),
              "f": [b.detach().cpu().clone() for b in self._state_buffers()],
              "mom": [m.detach().cpu().clone() for m in self.mom],
              "tau": self.tau_state.detach().cpu().clone() if self.powerlaw else None,
              "time": self.lb.time[None]}
        return ck

    def restore(self, ck):
        """Resume a run from checkpoint() output (or its torch.load()): binds
        this solver's buffers, loads the state and leaves the run live, as
        begin() does; continue with run(n) / a Batch, then finish()."""
        if not isinstance(ck, dict) or ck.get("format") != self.CHECKPOINT_FORMAT:
            raise ValueError("not a fused-solver checkpoint")
        if ck["plan"] != self._fingerprint():
            raise ValueError(f"checkpoint is for another lattice or plan: {ck['plan']} != {self._fingerprint()}")
        if getattr(self, "_live", False):
            raise RuntimeError("restore() on a live run; finish() it first")
        self._bind()
        for dst, src in zip(self._state_buffers(), ck["f"]):
            if dst.shape != src.shape or dst.dtype != src.dtype:
                raise ValueError("checkpoint buffer shape or type differs")
            dst.copy_(src)
        for dst, src in zip(self.mom, ck["mom"]):
            dst.copy_(src)
        if self.powerlaw:
            self.tau_state.copy_(ck["tau"])
        A.call("lbm_plan_set_parity", self._plan, int(ck["parity"]))
        self.lb.time[None] = ck["time"]
        self.lb._fused_owner = self
        self._live = True

    def parity_now(self):
        """0: the live state is in the first buffer (f2's storage for fp32)."""
        par = ctypes.c_int32()
        A.call("lbm_plan_get_parity", self._plan, ctypes.byref(par))
        return par.value

    def step(self, n=1, forces=False):
        """n reference steps (n calls of lbm_solve()) + the next moment prologue.

        forces=True also returns the force on the solid obstacles after each
        step's collision (momentum exchange on bounce-back links into mask=-1
        nodes): an (n, 2) float64 CUDA tensor, row s = step s+1."""
        n = int(n)
        if n <= 0:
            return None
        self.begin()
        series = None
        if forces:
            links = self.solid_links()
            series = torch.zeros((n, 2), dtype=torch.float64, device=self.lb.device)
            lp, ln = ctypes.c_void_p(links.data_ptr()), links.shape[0]
            s = stream_handle()
            A.call("lbm_plan_momentum_exchange", self._plan, lp, ln,
                   ctypes.c_void_p(series.data_ptr()), s)
            if n > 1:
                A.call("lbm_plan_run_monitored", self._plan, n - 1, lp, ln,
                       ctypes.c_void_p(series[1:].data_ptr()), s)
        elif n > 1:
            self.run(n - 1)
        self.finish()
        if self.sc is not None:  # the Shan-Chen driver advances LBField.time (lbm.py:150-151)
            self.lb.time[None] = self.lb.time[None] + n
        return series

    def solid_links(self):
        """(m, 2) int32 device tensor of (j*pitch + i, k): colliding node and
        outgoing link k whose neighbour (i + cx_k, j + cy_k) is a solid node
        reached through a bounce-back link."""
        if getattr(self, "_solid_links", None) is not None:
            return self._solid_links
        lb = self.lb
        code = self.compiled.code.astype(np.int64)
        nx, ny = lb.NX, lb.NY
        solid = np.pad(lb.mask.arr == -1, 1, constant_values=False)  # outside: not solid
        cx = (0, 1, 0, -1, 0, 1, -1, -1, 1)
        cy = (0, 0, 1, 0, -1, 1, 1, -1, -1)
        opp = (0, 3, 4, 1, 2, 7, 8, 5, 6)
        rows = []
        active = (code & A.CODE_ACTIVE) != 0
        for kp in range(1, 9):
            k = opp[kp]
            sel = active & (((code >> (kp - 1)) & 1) == 1) & \
                solid[1 + cx[k]:1 + cx[k] + nx, 1 + cy[k]:1 + cy[k] + ny]
            ii, jj = np.nonzero(sel)  # i-major, the order of the node grid
            rows.append(np.stack([jj * lb.pitch + ii, np.full_like(ii, k)], 1))
        links = np.concatenate(rows).astype(np.int32) if rows else np.zeros((0, 2), np.int32)
        t = torch.as_tensor(links if links.size else np.zeros((1, 2), np.int32), device=lb.device)
        self._solid_links = t[:links.shape[0]] if links.size else t[:0]
        self._solid_links_host = links
        return self._solid_links

    def reduce_moments(self):
        """FP64 (sum f, sum f cx, sum f cy) over colliding nodes of the live
        fused state (call between begin() and finish())."""
        scratch = torch.empty(int(A.load().lbm_reduce_scratch_doubles()), dtype=torch.float64,
                              device=self.lb.device)
        out = torch.empty(3, dtype=torch.float64, device=self.lb.device)
        A.call("lbm_plan_reduce_moments", self._plan, ctypes.c_void_p(scratch.data_ptr()),
               ctypes.c_void_p(out.data_ptr()), stream_handle())
        return out
