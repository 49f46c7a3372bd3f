"""ctypes driver for the CPU oracle (test infrastructure, not product).

Replays a *case description* — the lattice, mask, boundary groups in
application order, collision/fluid-model/Shan-Chen parameters and initial
moments — through the C++ restatement in ``lbm_oracle.cpp``, calling the
stages in the reference's step order:

* standard   ``cases/Circular cylinder.py:182-193``
* powerlaw   ``cases/Power Law Fluid.py:160-173``
* shanchen   ``cases/Bubble or two-phase separation.py:197-212``

and then the moment prologue of the next step (the comparison point).

A case description is ``(meta, arrays)``: ``meta`` is the JSON dict written
by ``tests/golden/make_golden.py`` (and emitted by the product's
``describe()``), ``arrays`` holds ``mask``, ``init_rho``, ``init_vel`` and one
``g_<name>`` index array per boundary condition.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

_I32P = ctypes.POINTER(ctypes.c_int32)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        vp, i64, d, i = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_int
        sig = {
            "orc_create": ([i, i, i], vp), "orc_destroy": ([vp], None),
            "orc_field": ([vp, ctypes.c_char_p, ctypes.POINTER(i64)], vp),
            "orc_error": ([vp], i),
            "orc_mask_circle": ([vp, d, d, d], None), "orc_mask_rect": ([vp, d, d, d, d], None),
            "orc_neighbor_classify": ([vp], None), "orc_init_lbm": ([vp, vp, i64], None),
            "orc_density": ([vp, vp, i64], None), "orc_pressure": ([vp, vp, i64, i, d], None),
            "orc_force_density": ([vp, vp, i64], None), "orc_velocity": ([vp, vp, i64], None),
            "orc_bgk_init_tau": ([vp, vp, i64, d], None), "orc_bgk_shear_rate": ([vp, vp, i64], None),
            "orc_bgk_relaxation_time": ([vp, vp, i64, i, d, d, d, d, d], None),
            "orc_bgk_apply": ([vp, vp, i64], None),
            "orc_trt_init_tau": ([vp, vp, i64, d, d], None), "orc_trt_shear_rate": ([vp, vp, i64], None),
            "orc_trt_relaxation_time": ([vp, vp, i64, i, d, d, d, d, d, d], None),
            "orc_trt_apply": ([vp, vp, i64], None),
            "orc_mrt_init_tau": ([vp, vp, i64, d, d, d, d], None),
            "orc_mrt_shear_rate": ([vp, vp, i64], None),
            "orc_mrt_relaxation_time": ([vp, vp, i64, i, d, d, d, d, d], None),
            "orc_mrt_apply": ([vp, vp, i64], None),
            "orc_sc_update_psi": ([vp, vp, i64, vp], None), "orc_sc_force": ([vp, vp, i64, d], None),
            "orc_psi_periodic_lr": ([vp], None), "orc_psi_periodic_bt": ([vp], None),
            "orc_psi_fixed": ([vp, vp, i64, d], None), "orc_psi_open": ([vp, vp, i64, i, i], None),
            "orc_get_psi": ([vp, d, d, i], d),
            "orc_bc_periodic": ([vp, vp, i64], None), "orc_bc_inside": ([vp, vp, i64], None),
            "orc_bc_bounceback": ([vp, vp, i64], None),
            "orc_bc_velocity_bb": ([vp, vp, i64, i, vp], None),
            "orc_bc_velocity_eq": ([vp, vp, i64, i, vp], None),
            "orc_bc_velocity_neem": ([vp, vp, i64, i, vp], None),
            "orc_bc_pressure_abc": ([vp, vp, i64, i, d], None),
            "orc_bc_pressure_neem": ([vp, vp, i64, i, d], None),
            "orc_bc_open_neumann": ([vp, vp, i64, i], None),
            "orc_bc_open_conv1": ([vp, vp, i64, i], None),
            "orc_bc_open_conv2": ([vp, vp, i64, i, d, vp], None),
            "orc_bc_open_extrap": ([vp, vp, i64, i], None),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


EOS_KIND = {"sc": 0, "vdw": 1, "rk": 2, "pr": 3, "cs": 4}
# open psi boundaries (SCBoundaryCondition.py:19-110) -> orc_psi_open kind
PSI_OPEN = {"open_neumann_psi": 0, "open_conv1_psi": 1, "open_conv2_psi": 2, "open_extrap_psi": 3}


def eos_vector(psi):
    """[kind, params] -> the 8 doubles the C side takes."""
    kind = psi[0]
    if kind == "sc":
        return np.array([0, 0, 0, 0, 0, float(psi[1]), 0, 0], np.float64)
    p = psi[1]
    return np.array([EOS_KIND[kind], p.get("a") or 0.0, p.get("b") or 0.0, p.get("R", 1.0),
                     p.get("G", 1.0), 0.0, p.get("omega", 0.0) or 0.0,
                     p.get("temperature_cr") or 1.0], np.float64)


FIELD_SHAPES = {
    "f": (9,), "f2": (9,), "vel": (2,), "body_force": (2,), "SCforce": (2,), "diag": (9,),
    "neighbor": (9, 2),
}


class Oracle:
    """One lattice of the CPU restatement, fields exposed as numpy views in
    the reference's index order ``[i, j, ...]``."""

    def __init__(self, nx, ny, dbl=False):
        self.L = lib()
        self.nx, self.ny, self.dbl = nx, ny, bool(dbl)
        self.dtype = np.float64 if dbl else np.float32
        self.h = self.L.orc_create(nx, ny, int(bool(dbl)))

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field(self, name):
        n = ctypes.c_int64()
        ptr = self.L.orc_field(self.h, name.encode(), ctypes.byref(n))
        if not ptr:
            raise KeyError(name)
        dt = np.int32 if name in ("mask", "neighbor") else self.dtype
        buf = (ctypes.c_char * (n.value * np.dtype(dt).itemsize)).from_address(ptr)
        a = np.frombuffer(buf, dtype=dt, count=n.value)
        if name == "psi":
            return a.reshape(self.nx + 2, self.ny + 2)
        if name in ("M", "M_inverse"):
            return a.reshape(9, 9)
        if name in ("weights", "gravity"):
            return a
        return a.reshape((self.nx, self.ny) + FIELD_SHAPES.get(name, ()))

    @staticmethod
    def _g(group):
        g = np.ascontiguousarray(group, dtype=np.int32).reshape(-1, 2)
        return g, g.ctypes.data, g.shape[0]

    def call(self, name, group, *args):
        g, p, n = self._g(group)
        getattr(self.L, "orc_" + name)(self.h, p, n, *args)

    def error(self):
        return self.L.orc_error(self.h)


def _fluid_model_args(meta):
    fm = meta["fluid_model"]
    if fm[0] == "newtonian":
        return 0, float(fm[1]), 0.0, 1.0
    return 1, 0.0, float(fm[1]), float(fm[2])


class Run:
    """A prepared oracle lattice: ``step(n)`` runs n reference steps,
    ``finish()`` runs the next moment prologue and returns the fields."""

    def __init__(self, o, step, moments, extract):
        self.o, self._step, self._moments, self._extract = o, step, moments, extract

    def step(self, n=1):
        for _ in range(int(n)):
            self._step()

    def finish(self):
        self._moments()
        out = self._extract()
        self.o.close()
        return out


def replay(meta, arrays, steps=None, nthreads=None):
    """Run a case description through the oracle; returns a dict of fields
    at the comparison point (after the moment prologue of step steps+1)."""
    r = prepare(meta, arrays, nthreads)
    r.step(int(meta["steps"] if steps is None else steps))
    return r.finish()


def prepare(meta, arrays, nthreads=None):
    """Set a case description up in the oracle (mask, neighbor table,
    collision state, initial populations) and return a Run."""
    if nthreads is not None:
        os.environ["OMP_NUM_THREADS"] = str(nthreads)
    nx, ny = int(meta["NX"]), int(meta["NY"])
    dbl = meta.get("fp", "f32") == "f64"
    o = Oracle(nx, ny, dbl)
    dt = o.dtype
    mask = o.field("mask")
    mask[...] = arrays["mask"]
    o.L.orc_neighbor_classify(o.h)
    o.field("gravity")[...] = np.asarray(meta.get("gravity", [0.0, 0.0]), np.float64)

    bcs = meta["bcs"]
    groups = {b["name"]: np.ascontiguousarray(arrays["g_" + b["name"]], np.int32).reshape(-1, 2)
              for b in bcs}
    fluid = groups[bcs[0]["name"]]
    rho = o.field("rho")
    vel = o.field("vel")
    rho[...] = np.asarray(arrays["init_rho"], dt)
    vel[...] = np.asarray(arrays["init_vel"], dt)

    coll = meta["collision"]
    model = coll["model"]
    lo, hi = float(coll["tau_min"]), float(coll["tau_max"])
    nu = float(coll["nu"][0])
    if model == "bgk":
        o.call("bgk_init_tau", fluid, nu)
    elif model == "trt":
        o.call("trt_init_tau", fluid, nu, float(coll["magic"][0]))
    else:
        M = o.field("M").astype(np.float64)
        o.field("M_inverse")[...] = np.linalg.inv(M).astype(dt)
        o.call("mrt_init_tau", fluid, nu, float(coll["nu_bulk"][0]), lo, hi)
        if coll.get("mrt_diag") is not None:
            d = o.field("diag")
            d[fluid[:, 0], fluid[:, 1]] = np.asarray(coll["mrt_diag"], np.float64).astype(dt)

    sc = meta.get("sc")
    eos = None
    if sc is not None:
        o.field("T")[...] = np.asarray(arrays["T"], dt) if "T" in arrays else dt(meta.get("T", 1.0))
        eos = eos_vector(sc["psi"])
    o.call("init_lbm", fluid)

    fk, fnu, fm_m, fm_n = _fluid_model_args(meta)
    kind = meta["step_kind"]

    uvels = {}
    for b in bcs:
        if "velocity" in b and b["kind"].startswith("velocity"):
            g = groups[b["name"]]
            if "velocity_per_node" in arrays.get("_extra", {}):
                pass
            v = np.asarray(b["velocity"], np.float64).astype(dt)
            key = "u_" + b["name"]
            per = arrays[key] if key in arrays else np.tile(v, (g.shape[0], 1))
            uvels[b["name"]] = np.ascontiguousarray(np.asarray(per, dt).reshape(-1, 2))

    def apply_bcs():
        for b in bcs:
            g = groups[b["name"]]
            k = b["kind"]
            if k == "fluid":
                continue
            if k == "periodic":
                o.call("bc_periodic", g)
            elif k == "inside":
                o.call("bc_inside", g)
            elif k == "bounceback":
                o.call("bc_bounceback", g)
            elif k in ("velocity_eq", "velocity_neem", "velocity_bb"):
                u = uvels[b["name"]]
                o.call("bc_" + k, g, int(b["direction"]), u.ctypes.data)
            elif k in ("pressure_neem", "pressure_abc"):
                o.call("bc_" + k, g, int(b["direction"]), float(b["rho"]))
            elif k in ("open_neumann", "open_conv1", "open_extrap"):
                o.call("bc_" + k, g, int(b["direction"]))
            elif k == "open_conv2":
                o.call("bc_open_conv2", g, int(b["direction"]), float(sc["g_coh"]), eos.ctypes.data)
            else:
                raise ValueError(f"unknown boundary kind {k}")

    psi_groups = {pb["name"]: np.ascontiguousarray(arrays["g_" + pb["name"]], np.int32).reshape(-1, 2)
                  for pb in meta.get("psi_bcs", []) if isinstance(pb, dict)}

    def apply_psi_bcs():
        for pb in meta.get("psi_bcs", []):
            if pb == "periodic_lr":
                o.L.orc_psi_periodic_lr(o.h)
            elif pb == "periodic_bt":
                o.L.orc_psi_periodic_bt(o.h)
            elif isinstance(pb, dict) and pb["kind"] == "fixed":
                o.call("psi_fixed", psi_groups[pb["name"]], float(pb["value"]))
            elif isinstance(pb, dict) and pb["kind"] in PSI_OPEN:
                o.call("psi_open", psi_groups[pb["name"]], PSI_OPEN[pb["kind"]], int(pb["direction"]))
            else:
                raise ValueError(pb)

    def moments():
        o.call("density", fluid)
        o.call("pressure", fluid, int(sc is not None), float(sc["g_coh"]) if sc else 0.0)
        if sc is not None:
            o.call("sc_update_psi", fluid, eos.ctypes.data)
            apply_psi_bcs()
            o.call("sc_force", fluid, float(sc["g_coh"]))
        o.call("force_density", fluid)
        o.call("velocity", fluid)

    def collide():
        if kind == "powerlaw":
            o.call(model + "_shear_rate", fluid)
            if model == "trt":
                o.call("trt_relaxation_time", fluid, fk, fnu, fm_m, fm_n, float(coll["magic"][0]), lo, hi)
            else:
                o.call(model + "_relaxation_time", fluid, fk, fnu, fm_m, fm_n, lo, hi)
        o.call(model + "_apply", fluid)

    def step():
        moments()
        collide()
        apply_bcs()

    return Run(o, step, moments, lambda: _extract(o, model, sc))


def _extract(o, model, sc):
    out = {}
    for name in ("f", "f2", "rho", "total_rho", "vel", "body_force", "total_pressure", "shear_rate",
                 "mask", "neighbor"):
        out[name] = o.field(name).copy()
    out["pressure"] = out.pop("total_pressure")
    if model == "bgk":
        out["tau"] = o.field("tau").copy()
    elif model == "trt":
        out["tau_sym"] = o.field("tau_sym").copy()
        out["tau_antisym"] = o.field("tau_antisym").copy()
    else:
        out["diag"] = o.field("diag").copy()
    if sc is not None:
        out["psi"] = o.field("psi").copy()
        out["sc_force"] = o.field("SCforce").copy()
    out["error"] = o.error()
    return out
