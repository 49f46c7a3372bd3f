"""Many lattices advanced together: a thin owner of an LbmBatch (C ABI).

A member is a FusedSolver whose state is live on the device (begin() has
run: the first step is done with the per-stage kernels, exactly as
FusedSolver.step does).  Batch.run(n) then advances every member n steps,
one persistent launch per kernel group per step (see lbm_batch_run in
lbm_gb300.h); FusedSolver.finish() ends a member's run as usual.  So for one
solver, ``begin(); batch.run(n - 1); finish()`` is ``step(n)``.

Drag/lift monitors: ``add(solver, monitor_steps=m)`` records the momentum
exchanged on the member's solid links after its first step and after every
batched step, up to m rows; ``forces(slot)`` returns them as an (rows, 2)
float64 CUDA tensor, the series FusedSolver.step(n, forces=True) returns.
"""
import ctypes

import numpy as np
import torch

from . import _capi as A
from .lbm import stream_handle


class Batch:
    def __init__(self, graphs=True, solo_nodes=None, sc_rows=None, lean_form=None):
        """solo_nodes: members of at least this many nodes run their own
        single-lattice step inside each batched step (lbm_batch_set_solo);
        None keeps the library default, 0 packs every member.  sc_rows: rows
        per Shan-Chen strip (8, 16, 32; None chooses from the batch).
        lean_form: kernel form of the plain segments (lbm_batch_set_lean_form:
        0 one pass per tile, 1 and 2 cp.async-pipelined; None keeps 0)."""
        h = ctypes.c_void_p()
        A.call("lbm_batch_create", ctypes.byref(h))
        self._h = h
        self.graphs = bool(graphs)
        A.call("lbm_batch_set_graph", self._h, 1 if self.graphs else 0)
        if solo_nodes is not None:
            A.call("lbm_batch_set_solo", self._h, int(solo_nodes))
        if sc_rows is not None:
            A.call("lbm_batch_set_sc_rows", self._h, int(sc_rows))
        if lean_form is not None:
            A.call("lbm_batch_set_lean_form", self._h, int(lean_form))
        self.members = {}  # slot -> (solver, monitor tensors or None)

    @staticmethod
    def prepare(solver, monitor_steps=0):
        """Begin `solver`'s run if needed and, for monitor_steps > 0, record its
        first-step drag/lift row; returns the monitor tensors (or None) for
        add().  Runs on the current stream, so a builder thread may prepare
        members on its own stream."""
        if not getattr(solver, "_live", False):
            solver.begin()
        if not monitor_steps:
            return None
        links = solver.solid_links()
        series = torch.zeros((int(monitor_steps), 2), dtype=torch.float64, device=solver.lb.device)
        count = torch.ones(1, dtype=torch.int32, device=solver.lb.device)
        A.call("lbm_plan_momentum_exchange", solver._plan, ctypes.c_void_p(links.data_ptr()),
               links.shape[0], ctypes.c_void_p(series.data_ptr()), stream_handle())
        return (links, series, count)

    def add(self, solver, monitor_steps=0, prepared=None):
        """Join `solver` (beginning its run if needed); returns its slot.
        `prepared`: the result of Batch.prepare(solver, monitor_steps)."""
        mon = prepared if prepared is not None else self.prepare(solver, monitor_steps)
        slot = ctypes.c_int32()
        masks = None
        if solver.sc is None:
            masks = np.ascontiguousarray(np.asarray(solver.compiled.lane_mask, np.uint32))
        A.call("lbm_batch_add", self._h, solver._plan,
               None if masks is None else masks.ctypes.data_as(ctypes.c_void_p), ctypes.byref(slot))
        if mon is not None:
            links, series, count = mon
            A.call("lbm_batch_monitor", self._h, slot.value, ctypes.c_void_p(links.data_ptr()),
                   links.shape[0], ctypes.c_void_p(series.data_ptr()), ctypes.c_void_p(count.data_ptr()),
                   series.shape[0])
        self.members[slot.value] = (solver, mon)
        return slot.value

    def remove(self, slot):
        """Leave the batch; returns the solver (its state stays live).  Steps
        already queued still compute the member: work on the current stream
        after this call (finish(), reading its fields) follows them."""
        A.call("lbm_batch_remove", self._h, int(slot))
        solver, _ = self.members.pop(int(slot))
        return solver

    def run(self, nsteps):
        A.call("lbm_batch_run", self._h, int(nsteps), stream_handle())

    def forces(self, slot):
        """(rows recorded, 2) float64 drag/lift series of a monitored member."""
        _, mon = self.members[int(slot)]
        if mon is None:
            raise ValueError(f"member {slot} has no monitor")
        _, series, count = mon
        n = min(int(count.item()), series.shape[0])
        return series[:n]

    def info(self):
        m, t, g = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32()
        A.call("lbm_batch_info", self._h, ctypes.byref(m), ctypes.byref(t), ctypes.byref(g))
        return {"members": m.value, "tiles": t.value, "groups": g.value}

    def close(self):
        if self._h is not None:
            A.load().lbm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
