"""Build a case description (fixture meta + arrays) through the drop-in API.

The same description feeds the oracle (oracle.oracle.replay), so a GPU run
and an oracle run see identical groups, parameters and initial moments.
Also builds the cylinder-channel workloads of the benchmark at any size.
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "taichi-lbm_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
if PKG not in sys.path:
    sys.path.insert(0, PKG)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def load_fixture(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    arrays = {k: d[k] for k in d.files}
    meta = json.loads(str(arrays.pop("meta")))
    return meta, arrays


def fixture_names():
    """Fixtures of the single-component step (the multi-component ones, mc_*,
    and the immersed-boundary ones, ibm_*, have their own oracles and tests)."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.endswith(".npz") and not f.startswith(("mc_", "ibm_")))


def _member_fn_halo(nodes, nx, ny):
    """Predicate over psi coordinates (-1..NX, -1..NY)."""
    sel = np.zeros((nx + 2, ny + 2), bool)
    if nodes.size:
        sel[nodes[:, 0] + 1, nodes[:, 1] + 1] = True
    return lambda i, j: sel[np.asarray(i) + 1, np.asarray(j) + 1]


def _member_fn(nodes, nx, ny):
    sel = np.zeros((nx, ny), bool)
    if nodes.size:
        sel[nodes[:, 0], nodes[:, 1]] = True
    return lambda i, j: sel[i, j]


def build_from_case(tl, meta, arrays, value_fn_inlet=False):
    """Returns (lb, me, coll, be, sc, bsc) built through the drop-in API."""
    nx, ny = int(meta["NX"]), int(meta["NY"])
    lb = tl.LBField(meta["name"], nx, ny, 1)
    lb.keep_init_snapshot = True
    lb.mask.from_numpy(arrays["mask"])
    if any(meta.get("gravity", [0, 0])):
        lb.set_gravity(meta["gravity"])
    cls = tl.BoundaryClassifier((nx, ny))
    be = tl.BoundaryEngine()
    bcs = meta["bcs"]
    fluid_nodes = arrays["g_" + bcs[0]["name"]]
    fluid = None
    inlet_batch = []
    for b in bcs:
        nodes = arrays["g_" + b["name"]]
        spec = tl.BoundarySpec(geometry_fn=_member_fn(nodes, nx, ny))
        k = b["kind"]
        d = b.get("direction")
        if k == "fluid":
            bc = tl.FluidBoundary(spec=spec)
        elif k == "periodic":
            bc = tl.PeriodicAllBoundary(spec=spec)
        elif k == "inside":
            bc = tl.InsideBoundary(spec=spec)
        elif k == "bounceback":
            bc = tl.BounceBackWall(spec=spec)
        elif k in ("velocity_eq", "velocity_neem", "velocity_bb"):
            cls_ = {"velocity_eq": tl.VelocityEquilibrium, "velocity_neem": tl.VelocityNEEM,
                    "velocity_bb": tl.VelocityBB}[k]
            if value_fn_inlet and k == "velocity_eq" and b["name"].startswith("inlet"):
                inlet_batch.append((nodes, b["velocity"]))
                continue
            bc = cls_(spec=spec, velocity_value=b["velocity"], direction=d)
        elif k == "pressure_neem":
            bc = tl.PressureNEEM(spec=spec, rho_value=b["rho"], direction=d)
        elif k == "pressure_abc":
            bc = tl.PressureABC(spec=spec, rho_value=b["rho"], direction=d)
        elif k == "open_neumann":
            bc = tl.OpenNeumann(spec=spec, direction=d)
        elif k == "open_conv1":
            bc = tl.OpenConvective1order(spec=spec, direction=d)
        elif k == "open_extrap":
            bc = tl.OpenExtrapolation(spec=spec, direction=d)
        elif k == "open_conv2":
            bc = tl.OpenConvective2order(spec=spec, direction=d)
        else:
            raise ValueError(k)
        if inlet_batch and not b["name"].startswith("inlet"):
            _add_value_fn_inlet(tl, be, cls, inlet_batch, nx, ny)
            inlet_batch = []
        bc.precompute(classifier=cls)
        be.add_boundary_condition(b["name"], bc)
        if k == "fluid" and fluid is None:
            fluid = bc
    if inlet_batch:
        _add_value_fn_inlet(tl, be, cls, inlet_batch, nx, ny)
    lb.neighbor_classify()
    me = tl.MacroscopicEngine(fluid.group)
    coll = make_collision(tl, meta, lb, fluid.group)
    lb.rho.from_numpy(np.asarray(arrays["init_rho"], np.float32)[:, :, None])
    lb.vel.from_numpy(np.asarray(arrays["init_vel"], np.float32))
    sc = bsc = None
    if meta.get("sc"):
        s = meta["sc"]
        psi = s["psi"]
        if psi[0] == "sc":
            model = tl.SC_psi(rho0=psi[1])
        else:
            model = {"cs": tl.CS_psi, "vdw": tl.vdW_psi, "rk": tl.RK_psi, "pr": tl.PR_psi}[psi[0]](psi[1])
        sc = tl.ShanChenForceC1({"lb_field": lb, "g_coh": s["g_coh"], "group": fluid.group,
                                 "psi": model})
        lb.sc_field = sc
        bsc = tl.BoundaryEngineSC()
        psi_kinds = {"open_neumann_psi": tl.OpenNeumannPsi, "open_conv1_psi": tl.OpenConvective1orderPsi,
                     "open_conv2_psi": tl.OpenConvective2orderPsi, "open_extrap_psi": tl.OpenExtrapolationPsi}
        for pb in meta.get("psi_bcs", []):
            if isinstance(pb, dict) and pb["kind"] == "fixed":  # FixedPsi on a recorded group
                fp = tl.FixedPsi(spec=tl.BoundarySpec(geometry_fn=_member_fn(arrays["g_" + pb["name"]], nx, ny)),
                                 psi_value=pb["value"])
                fp.precompute(classifier=cls)
                bsc.add_boundary_condition(pb["name"], fp)
                continue
            if isinstance(pb, dict):  # an open psi boundary on psi coordinates
                spec = tl.BoundarySpec(geometry_fn=_member_fn_halo(arrays["g_" + pb["name"]], nx, ny))
                ob = psi_kinds[pb["kind"]](spec, pb["direction"])
                ob.precompute(classifier=tl.BoundaryClassifier((nx + 2, ny + 2), offset=(-1, -1)))
                bsc.add_boundary_condition(pb["name"], ob)
                continue
            bsc.add_boundary_condition(pb, tl.PeriodicPsi_LR() if pb == "periodic_lr" else tl.PeriodicPsi_BT())
        lb.T.from_numpy(np.asarray(arrays["T"], np.float32) if "T" in arrays
                        else np.full((nx, ny), meta.get("T", 1.0), np.float32))
    lb.init_LBM(coll, fluid.group)
    return lb, me, coll, be, sc, bsc


def _add_value_fn_inlet(tl, be, cls, batch, nx, ny):
    nodes = np.concatenate([n for n, _ in batch])
    table = np.zeros((nx, ny, 2), np.float32)
    for n, v in batch:
        table[n[:, 0], n[:, 1]] = np.asarray(v, np.float32)
    spec = tl.BoundarySpec(geometry_fn=_member_fn(nodes, nx, ny),
                           value_fn=lambda i, j: (table[i, j, 0], table[i, j, 1]))
    bc = tl.VelocityEquilibrium(spec=spec, velocity_value=[0.0, 0.0], direction=3)
    bc.precompute(classifier=cls)
    be.add_boundary_condition("inlet", bc)


def make_collision(tl, meta, lb, group):
    c = meta["collision"]
    fm = meta["fluid_model"]
    fluid_model = tl.NewtonianFluid(nu=fm[1]) if fm[0] == "newtonian" else tl.PowerLawFluid(fm[1], fm[2])
    params = {"group": group, "fluid_model": fluid_model, "NX": lb.NX, "NY": lb.NY,
              "num_components": 1, "shearviscosity": c["nu"]}
    model = c["model"]
    if model == "bgk":
        coll = tl.BGKCollision(params)
    elif model == "trt":
        params["magic"] = c["magic"]
        coll = tl.TRTCollision(params)
    else:
        params["bulkviscosity"] = c["nu_bulk"]
        params["tau_clamp"] = (c["tau_min"], c["tau_max"])
        coll = tl.MRTCollision(params)
        if c.get("mrt_diag") is not None:
            coll.set_rates(c["mrt_diag"])
    coll.tau_min, coll.tau_max = c["tau_min"], c["tau_max"]
    return coll


def run_staged(lb, me, coll, be, sc, bsc, kind, steps):
    """The reference's lbm_solve() composition, step by step, then the
    moment prologue of the next step."""
    for _ in range(steps):
        me.density(lb)
        me.pressure(lb)
        if kind == "shanchen":
            sc.update_psi(lb)
            bsc.apply_boundary_conditions(lb)
            sc.cau_SCforce(lb)
        me.force_density(lb)
        me.velocity(lb)
        if kind == "powerlaw":
            coll.shear_rate(lb)
            coll.relaxation_time(lb)
        coll.apply(lb)
        be.apply_boundary_conditions(lb)
        if kind == "shanchen":
            me.time_updata(lb)
    me.density(lb)
    me.pressure(lb)
    if kind == "shanchen":
        sc.update_psi(lb)
        bsc.apply_boundary_conditions(lb)
        sc.cau_SCforce(lb)
    me.force_density(lb)
    me.velocity(lb)


def fields_of(lb, coll=None):
    out = {"f": lb.f.to_numpy()[:, :, 0, :], "f2": lb.f2.to_numpy()[:, :, 0, :],
           "rho": lb.rho.to_numpy()[:, :, 0], "vel": lb.vel.to_numpy(),
           "pressure": lb.total_pressure.to_numpy()}
    if lb.sc_field is not None:
        out["psi"] = lb.sc_field.psi_field.to_numpy()[:, :, 0]
    return out


def rel_err(a, b):
    """max |a - b| / max |b| over the field (u -> 0 at walls, so a per-node
    relative error is meaningless there)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / (scale if scale > 0 else 1.0))


from taichi_lbm.workloads import cylinder_channel  # noqa: E402,F401


def describe(lb, coll, be, steps, step_kind="standard", fp="f32"):
    """Case description of a drop-in setup, for oracle.replay."""
    meta = {"name": lb.name, "NX": lb.NX, "NY": lb.NY, "fp": fp, "steps": steps,
            "step_kind": step_kind, "gravity": [float(v) for v in np.asarray(lb.gravity_force)],
            "bcs": [], "sc": None, "psi_bcs": []}
    arrays = {"mask": lb.mask.to_numpy()}
    rho0, vel0, T0 = lb._init_snapshot
    arrays["init_rho"], arrays["init_vel"] = rho0, vel0
    kinds = {0: "fluid", 1: "velocity_bb", 2: "velocity_eq", 3: "velocity_neem", 4: "pressure_abc",
             5: "pressure_neem", 6: "open_neumann", 7: "open_conv1", 9: "open_extrap", 10: "periodic",
             11: "inside", 12: "bounceback"}
    for name, bc in be.boundary_conditions.items():
        d = {"name": name, "kind": kinds[bc.kind]}
        if getattr(bc, "direction", None):
            d["direction"] = bc.direction
        if hasattr(bc, "rho_value"):
            d["rho"] = float(bc.rho_value)
        if hasattr(bc, "velocity_value"):
            d["velocity"] = [float(v) for v in bc.velocity_array()]
            arrays["u_" + name] = bc.per_node_velocity_host()
        meta["bcs"].append(d)
        arrays["g_" + name] = bc.group.nodes
    fm = coll.fluid_model
    meta["fluid_model"] = (["newtonian", float(fm.nu)] if not hasattr(fm, "m")
                           else ["powerlaw", float(fm.m), float(fm.n)])
    c = {"model": {0: "bgk", 1: "trt", 2: "mrt"}[coll.model], "nu": [float(coll.nu[0])],
         "tau_min": float(coll.tau_min), "tau_max": float(coll.tau_max), "mrt_diag": None}
    if hasattr(coll, "magic"):
        c["magic"] = [float(coll.magic[0])]
    if hasattr(coll, "nu_bulk"):
        c["nu_bulk"] = [float(coll.nu_bulk[0])]
        nd = coll.group.nodes
        if nd.size:
            c["mrt_diag"] = [float(v) for v in coll._diag[:, nd[0, 1], nd[0, 0]].cpu().numpy()]
    meta["collision"] = c
    sc = lb.sc_field
    if sc is not None:
        kind = {0: "sc", 1: "vdw", 2: "rk", 3: "pr", 4: "cs"}[sc.psi.kind]
        meta["sc"] = {"g_coh": float(sc.g_coh),
                      "psi": ["sc", float(sc.psi.rho0)] if kind == "sc" else [kind, sc.psi.params]}
        meta["psi_bcs"] = ["periodic_lr", "periodic_bt"]
        meta["step_kind"] = "shanchen"
        arrays["T"] = T0
    return meta, arrays
