"""Autotuner for the batched and served step.

Chooses, by timing candidates on the device with CUDA events, the launch
shape the batch engine leaves open:

* nodes per thread V of a member (its row tile is 32·V nodes wide): 2 or 4
  for fp32 storage, 4 or 8 for the 16-bit shifted storages;
* rows per Shan-Chen strip (8, 16, 32): the strip tile's height;
* the solo threshold: members of at least that many nodes run their own
  single-lattice step inside the batched step rather than the packed tiles;
* the kernel form of the packed plain segments (one pass per tile, or a
  two- or three-stage cp.async pipeline per warp).

Results are kept in a table keyed by what decides them (collision model,
storage, power law, Shan-Chen, and the lattice's node count rounded to a
power of two), optionally saved as JSON, so a serving loop looks a request's
shape up without timing anything on its path.
"""
import json
import math
import os

import torch

V_CANDIDATES = {"fp32": (2, 4), "fp16s": (4, 8), "bf16s": (4, 8), "i16s": (4, 8)}
SC_ROWS = (8, 16, 32)
SOLO_CANDIDATES = (0, 1 << 18, 1 << 19, 1 << 20, 1 << 62)
LEAN_FORMS = (0, 1, 2)


def _elapsed_ms(fn, steps, warmup):
    st = torch.cuda.current_stream()
    fn(warmup)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    fn(steps)
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


class Autotuner:
    """Table of tuned launch shapes; `path` (JSON) persists it across runs."""

    def __init__(self, path=None, steps=40, warmup=5):
        self.path = path
        self.steps = int(steps)
        self.warmup = int(warmup)
        self.table = {}
        self.trials = []  # (key, candidate, ms per step) of every timing taken
        if path and os.path.exists(path):
            with open(path) as f:
                self.table = json.load(f)

    @staticmethod
    def key(model, storage, nodes, powerlaw=False, sc=False):
        bucket = 1 << max(0, int(math.ceil(math.log2(max(int(nodes), 1)))))
        return f"{model}/{storage}/{'pl' if powerlaw else 'nt'}/{'sc' if sc else 'plain'}/{bucket}"

    def save(self):
        if self.path:
            with open(self.path, "w") as f:
                json.dump(self.table, f, indent=1, sort_keys=True)

    def lookup(self, key, what, default=None):
        """Tuned value `what` for `key`, else that of the tuned entry with the
        same model/storage/fluid/kind and the nearest node-count bucket."""
        ent = self.table.get(key)
        if ent is not None and ent.get(what) is not None:
            return ent[what]
        prefix, _, bucket = key.rpartition("/")
        best, dist = default, None
        for k, e in self.table.items():
            p, _, b = k.rpartition("/")
            if p != prefix or e.get(what) is None or not b.isdigit():
                continue
            d = abs(math.log2(int(b)) - math.log2(int(bucket)))
            if dist is None or d < dist:
                best, dist = e[what], d
        return best

    # -------------------------------------------------------------- V
    def nodes_per_thread(self, key, storage, make_solver):
        """Best V for `key`: make_solver(V) returns a fresh FusedSolver of the
        shape; each candidate runs warmup + steps fused steps, timed."""
        hit = self.table.get(key, {}).get("V")
        if hit is not None:
            return int(hit)
        best, best_ms = None, None
        for V in V_CANDIDATES[storage]:
            s = make_solver(V)
            s.begin()
            ms = _elapsed_ms(s.run, self.steps, self.warmup)
            s.finish()
            del s
            self.trials.append((key, {"V": V}, ms))
            if best_ms is None or ms < best_ms:
                best, best_ms = V, ms
        self.table.setdefault(key, {})["V"] = best
        self.table[key]["V_ms"] = best_ms
        return best

    # -------------------------------------------------------------- batch
    def batch_shape(self, key, make_members, storage, graphs=True, sc=False, tune_v=True):
        """Best (V, solo_nodes, sc_rows) for a batch of the members
        make_members(V) returns (fresh FusedSolvers with V nodes per thread,
        or the default for V=None).  Each candidate is a new Batch over such
        members, timed over warmup + steps batched steps (the members'
        states advance; they are scratch).  Candidates: V over the storage's
        pair (tune_v), and the strip rows (Shan-Chen) or the solo thresholds
        times the lean kernel forms.  The chosen lean form is kept in the
        table entry (batch_kwargs passes it on)."""
        from .batch import Batch
        hit = self.table.get(key, {})
        if all(k in hit for k in ("V", "solo_nodes", "sc_rows")):
            return hit["V"], hit["solo_nodes"], hit["sc_rows"]
        shapes = ([(None, r, None) for r in SC_ROWS] if sc
                  else [(n, None, f) for n in SOLO_CANDIDATES for f in LEAN_FORMS])
        best, best_ms = None, None
        for V in (V_CANDIDATES[storage] if tune_v else (None,)):
            members = make_members(V)
            for solo, rows, form in shapes:
                b = Batch(graphs=graphs, solo_nodes=solo, sc_rows=rows, lean_form=form)
                for s in members:
                    b.add(s)
                ms = _elapsed_ms(b.run, self.steps, self.warmup)
                for slot in list(b.members):
                    b.remove(slot)
                b.close()
                self.trials.append((key, {"V": V, "solo_nodes": solo, "sc_rows": rows, "lean_form": form}, ms))
                if best_ms is None or ms < best_ms:
                    best, best_ms = (V, solo, rows, form), ms
            for s in members:
                s.finish()
            del members
        ent = self.table.setdefault(key, {})
        ent["V"] = None if best[0] is None else int(best[0])
        ent["solo_nodes"] = -1 if best[1] is None else int(best[1])
        ent["sc_rows"] = 0 if best[2] is None else int(best[2])
        ent["lean_form"] = 0 if best[3] is None else int(best[3])
        ent["batch_ms"] = best_ms
        return ent["V"], ent["solo_nodes"], ent["sc_rows"]

    def batch_kwargs(self, key):
        """Batch(...) keyword arguments from a tuned entry (empty if none)."""
        ent = self.table.get(key, {})
        kw = {}
        if ent.get("solo_nodes", -1) >= 0:
            kw["solo_nodes"] = int(ent["solo_nodes"])
        if ent.get("sc_rows", 0) > 0:
            kw["sc_rows"] = int(ent["sc_rows"])
        if ent.get("lean_form", 0) > 0:
            kw["lean_form"] = int(ent["lean_form"])
        return kw
