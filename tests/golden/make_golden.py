"""Generate golden fixtures by running the reference's own taichi_lbm source.

Runs only in a container that has the reference checkout; the fixtures it
writes (``tests/golden/*.npz``) are what travels.  Taichi itself cannot be
installed here, so ``_emu/`` supplies a serial stand-in for the Taichi runtime
(see ``_emu/taichi/__init__.py`` for exactly what it emulates); every line of
LBM arithmetic executed is the reference's.

Each case is built through the reference API the way its example scripts do
(``cases/Circular cylinder.py``, ``cases/contraction flow.py``,
``cases/Power Law Fluid.py``, ``cases/Bubble or two-phase separation.py``),
with boundary groups chosen so that no kernel indexes outside the lattice
(the example scripts' wall predicates read ``mask[-1, j]``, which is undefined
in Taichi and an error here).  A parabolic inlet, which the reference's
single-valued ``velocity_value`` cannot express, is built as one
VelocityEquilibrium boundary per inlet node.

After ``steps`` calls of the case's step function the driver runs the moment
prologue of the next step (density, pressure, [psi, SC force], force_density,
velocity) and records every field: that is the comparison point.

Usage:  python tests/golden/make_golden.py --ref PATH [case ...]
        (or TAICHI_LBM_REF=PATH in the environment instead of --ref)
"""
import argparse
import contextlib
import io
import json
import os
import sys
import time
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SEED = 20261203


def load_reference(ref_root, fp):
    sys.path.insert(0, os.path.join(HERE, "_emu"))
    sys.path.insert(0, ref_root)
    import taichi as ti
    ti.init(arch=ti.cpu, default_fp=ti.f64 if fp == "f64" else ti.f32)
    with contextlib.redirect_stdout(io.StringIO()):
        import taichi_lbm as tl
    return ti, tl


def parabola(j, ny, umax):
    """Channel profile with half-way walls at y=-1/2 and y=ny-1/2."""
    y = j + 0.5
    return 4.0 * umax * y * (ny - y) / (ny * ny)


class Case:
    """Case description recorded next to the fields (what the oracle replays)."""

    def __init__(self, name, nx, ny, fp):
        self.meta = {"name": name, "NX": nx, "NY": ny, "fp": fp, "bcs": [], "sc": None,
                     "psi_bcs": [], "gravity": [0.0, 0.0]}
        self.groups = {}

    def bc(self, name, kind, group, **kw):
        d = {"name": name, "kind": kind}
        d.update(kw)
        self.meta["bcs"].append(d)
        self.groups["g_" + name] = np.asarray(sorted(map(tuple, group)), np.int32).reshape(-1, 2)


def group_nodes(g):
    n = int(g.count[None])
    return [tuple(int(v) for v in g.group.arr[m]) for m in range(n)]


def build_channel(ti, tl, case, nx, ny, *, disc=None, rects=(), stream="periodic",
                  inlet=("eq_parabolic", 0.05), outlet=("pressure_neem", 1.0),
                  collision=("bgk", {}), nu=0.02, fluid_model=None, gravity=None,
                  tau_clamp=None, mrt_diag=None, init_u=None):
    """Channel with optional obstacles, walls on every lattice edge.

    stream: "periodic" = PeriodicAllBoundary over the fluid group followed by
    BounceBackWall over every fluid node with a missing link (the
    ``Circular cylinder.py`` pattern); "inside" = InsideBoundary over nodes
    with all links present plus the same BounceBackWall group (the
    ``contraction flow.py`` pattern without its out-of-range reads).
    """
    lb = tl.LBField(case.meta["name"], nx, ny, 1)
    if gravity is not None:
        lb.set_gravity(ti.Vector(list(gravity)))
        case.meta["gravity"] = list(gravity)
    be = tl.BoundaryEngine()
    cls = tl.BoundaryClassifier(ti.field(float, shape=(nx, ny)))
    if disc is not None:
        be.Mask_cricle_identify(lb, *disc)
        case.meta["disc"] = list(disc)
    for r in rects:
        be.Mask_rectangle_identify(lb, *r)
    case.meta["rects"] = [list(r) for r in rects]

    @ti.func
    def fluid_fn(i, j):
        return lb.mask[i, j] == 1

    def has_missing_link(i, j):
        flag = 0
        for k in range(9):
            ix2 = i - lb.c[k, 0]
            iy2 = j - lb.c[k, 1]
            if ix2 < 0 or ix2 > nx - 1 or iy2 < 0 or iy2 > ny - 1:
                flag = 1
            elif lb.mask[ix2, iy2] == -1:
                flag = 1
        return flag

    @ti.func
    def wall_fn(i, j):
        return lb.mask[i, j] == 1 and has_missing_link(i, j) == 1

    @ti.func
    def inside_fn(i, j):
        return lb.mask[i, j] == 1 and has_missing_link(i, j) == 0

    fluid = tl.FluidBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
    fluid.precompute(classifier=cls)
    be.add_boundary_condition("fluid", fluid)
    case.bc("fluid", "fluid", group_nodes(fluid.group))
    if stream == "periodic":
        per = tl.PeriodicAllBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
        per.precompute(classifier=cls)
        be.add_boundary_condition("periodic", per)
        case.bc("periodic", "periodic", group_nodes(per.group))
    else:
        ins = tl.InsideBoundary(spec=tl.BoundarySpec(geometry_fn=inside_fn))
        ins.precompute(classifier=cls)
        be.add_boundary_condition("inside", ins)
        case.bc("inside", "inside", group_nodes(ins.group))
    wall = tl.BounceBackWall(spec=tl.BoundarySpec(geometry_fn=wall_fn))
    wall.precompute(classifier=cls)
    be.add_boundary_condition("wall", wall)
    case.bc("wall", "bounceback", group_nodes(wall.group))

    kind, val = inlet
    if kind == "eq_parabolic":
        for j in range(ny):
            if lb.mask[0, j] != 1:
                continue
            u = parabola(j, ny, val)

            def make(jj):
                @ti.func
                def fn(i, j2):
                    return i == 0 and j2 == jj and lb.mask[i, j2] == 1
                return fn
            bc = tl.VelocityEquilibrium(spec=tl.BoundarySpec(geometry_fn=make(j)),
                                        velocity_value=ti.Vector([u, 0.0]), direction=3)
            bc.precompute(classifier=cls)
            be.add_boundary_condition(f"inlet{j}", bc)
            case.bc(f"inlet{j}", "velocity_eq", group_nodes(bc.group), direction=3,
                    velocity=[float(np.asarray(bc.velocity_value)[0]), 0.0])
    else:
        @ti.func
        def inlet_fn(i, j):
            return lb.mask[i, j] == 1 and i == 0
        spec = tl.BoundarySpec(geometry_fn=inlet_fn)
        cls_map = {"eq": tl.VelocityEquilibrium, "neem": tl.VelocityNEEM, "bb": tl.VelocityBB}
        kmap = {"eq": "velocity_eq", "neem": "velocity_neem", "bb": "velocity_bb"}
        bc = cls_map[kind](spec=spec, velocity_value=ti.Vector([val, 0.0]), direction=3)
        bc.precompute(classifier=cls)
        be.add_boundary_condition("inlet", bc)
        case.bc("inlet", kmap[kind], group_nodes(bc.group), direction=3,
                velocity=[float(np.asarray(bc.velocity_value)[0]), 0.0])

    okind, oval = outlet

    @ti.func
    def outlet_fn(i, j):
        return lb.mask[i, j] == 1 and i == nx - 1
    ospec = tl.BoundarySpec(geometry_fn=outlet_fn)
    if okind == "pressure_neem":
        bc = tl.PressureNEEM(spec=ospec, rho_value=oval, direction=1)
    elif okind == "pressure_abc":
        bc = tl.PressureABC(spec=ospec, rho_value=oval, direction=1)
    elif okind == "open_neumann":
        bc = tl.OpenNeumann(spec=ospec, direction=1)
    elif okind == "open_conv1":
        bc = tl.OpenConvective1order(spec=ospec, direction=1)
    elif okind == "open_extrap":
        bc = tl.OpenExtrapolation(spec=ospec, direction=1)
    else:
        raise ValueError(okind)
    bc.precompute(classifier=cls)
    be.add_boundary_condition("outlet", bc)
    kw = {"direction": 1}
    if okind.startswith("pressure"):
        kw["rho"] = float(oval)
    case.bc("outlet", okind, group_nodes(bc.group), **kw)

    lb.neighbor_classify()
    me = tl.MacroscopicEngine(fluid.group)
    coll = make_collision(ti, tl, case, lb, fluid.group, collision, nu, fluid_model,
                          tau_clamp, mrt_diag)

    # rho = 1, vel = init_u (default 0) on the fluid group, then f = f2 = feq
    for (i, j) in group_nodes(fluid.group):
        lb.rho[i, j, 0] = 1.0
        if init_u is not None:
            lb.vel[i, j] = ti.Vector([float(init_u(i, j)[0]), float(init_u(i, j)[1])])
    lb.init_LBM(coll, fluid.group)
    return lb, me, coll, be, None, None


def make_collision(ti, tl, case, lb, group, collision, nu, fluid_model, tau_clamp, mrt_diag):
    model, extra = collision
    if fluid_model is None:
        fm = tl.NewtonianFluid(nu=nu)
        case.meta["fluid_model"] = ["newtonian", nu]
    else:
        fm = tl.PowerLawFluid(fluid_model[0], fluid_model[1])
        case.meta["fluid_model"] = ["powerlaw", fluid_model[0], fluid_model[1]]
    params = {"group": group, "fluid_model": fm, "NX": lb.NX, "NY": lb.NY,
              "num_components": 1, "shearviscosity": [nu]}
    params.update(extra)
    cls = {"bgk": tl.BGKCollision, "trt": tl.TRTCollision, "mrt": tl.MRTCollision}[model]
    if tau_clamp is not None:
        # Taichi folds these attributes into f32 constants when it compiles.
        lo, hi = tau_clamp
    else:
        lo, hi = 0.5000001, 4.0
    ti_fp = ti.default_fp()
    if model == "mrt":
        # MRT clamps inside its constructor (initTau), so the clamp has to be
        # in place before it runs: patch the class default for this build.
        orig = tl.CollisionEngine.Collision.__init__

        def init_with_clamp(self, g, f):
            orig(self, g, f)
            self.tau_min = ti_fp(lo)
            self.tau_max = ti_fp(hi)
        tl.CollisionEngine.Collision.__init__ = init_with_clamp
        try:
            coll = cls(params)
        finally:
            tl.CollisionEngine.Collision.__init__ = orig
    else:
        coll = cls(params)
        coll.tau_min = ti_fp(lo)
        coll.tau_max = ti_fp(hi)
    if model == "trt" and tau_clamp is not None:
        pass
    if mrt_diag is not None:
        for (i, j) in group_nodes(group):
            coll.diag[i, j, 0] = ti.Vector(list(mrt_diag))
    case.meta["collision"] = {"model": model, "nu": [nu], "tau_min": lo, "tau_max": hi,
                              "magic": extra.get("magic"), "nu_bulk": extra.get("bulkviscosity"),
                              "mrt_diag": None if mrt_diag is None else [float(v) for v in mrt_diag]}
    return coll


def build_shanchen(ti, tl, case, nx, ny, *, eos, g_coh, rho_init, collision=("bgk", {}),
                   nu=0.5 / 3.0, T=1.0, gravity=None, fixed_psi=None, open_conv2=False, open_psi=None):
    """Fully periodic single-component Shan-Chen lattice (the two-phase
    separation pattern of ``Bubble or two-phase separation.py``).
    fixed_psi=(row, value): a FixedPsi on the nodes of that row, applied
    after the periodic psi boundaries.  open_conv2: an OpenConvective2order
    outlet (direction 1) on the last column, applied after the stream.
    open_psi=[(kind, row, direction), ...]: open psi boundaries on the psi
    nodes (i, row), 0 <= i < NX (halo rows allowed), classified over the
    psi grid; psi is then periodic in x only, and these follow."""
    lb = tl.LBField(case.meta["name"], nx, ny, 1)
    if gravity is not None:
        lb.set_gravity(ti.Vector(list(gravity)))
        case.meta["gravity"] = list(gravity)
    be = tl.BoundaryEngine()
    cls = tl.BoundaryClassifier(ti.field(float, shape=(nx, ny)))

    @ti.func
    def fluid_fn(i, j):
        return lb.mask[i, j] == 1
    fluid = tl.FluidBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
    fluid.precompute(classifier=cls)
    be.add_boundary_condition("fluid", fluid)
    case.bc("fluid", "fluid", group_nodes(fluid.group))
    per = tl.PeriodicAllBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
    per.precompute(classifier=cls)
    be.add_boundary_condition("stream", per)
    case.bc("stream", "periodic", group_nodes(per.group))
    if open_conv2:
        @ti.func
        def outlet_fn(i, j):
            return lb.mask[i, j] == 1 and i == nx - 1
        oc = tl.OpenConvective2order(spec=tl.BoundarySpec(geometry_fn=outlet_fn), direction=1)
        oc.precompute(classifier=cls)
        be.add_boundary_condition("outlet", oc)
        case.bc("outlet", "open_conv2", group_nodes(oc.group), direction=1)
    lb.neighbor_classify()
    me = tl.MacroscopicEngine(fluid.group)
    coll = make_collision(ti, tl, case, lb, fluid.group, collision, nu, None, None, None)

    kind = eos[0]
    if kind == "sc":
        psi = tl.SC_psi(rho0=eos[1])
        case.meta["sc"] = {"g_coh": g_coh, "psi": ["sc", eos[1]]}
    else:
        p = dict(eos[1])
        with contextlib.redirect_stdout(io.StringIO()):
            psi = {"cs": tl.CS_psi, "vdw": tl.vdW_psi, "rk": tl.RK_psi, "pr": tl.PR_psi}[kind](p)
        case.meta["sc"] = {"g_coh": g_coh, "psi": [kind, p]}
    lb.sc_field = tl.ShanChenForceC1({"lb_field": lb, "g_coh": g_coh, "group": fluid.group,
                                      "psi": psi})
    bsc = tl.BoundaryEngineSC()
    bsc.add_boundary_condition("periodicLR", tl.PeriodicPsi_LR())
    case.meta["psi_bcs"] = ["periodic_lr"]
    if open_psi:
        cls_psi = tl.BoundaryClassifier(ti.field(float, shape=(nx + 2, ny + 2), offset=(-1, -1)))
        kinds = {"open_neumann_psi": tl.OpenNeumannPsi, "open_conv1_psi": tl.OpenConvective1orderPsi,
                 "open_conv2_psi": tl.OpenConvective2orderPsi, "open_extrap_psi": tl.OpenExtrapolationPsi}
        for n_, (kind, row, direction) in enumerate(open_psi):
            def make(r):
                @ti.func
                def fn(i, j):
                    return j == r and i >= 0 and i < nx
                return fn
            ob = kinds[kind](tl.BoundarySpec(geometry_fn=make(row)), direction)
            ob.precompute(classifier=cls_psi)
            name = f"psi_{kind}_{n_}"
            bsc.add_boundary_condition(name, ob)
            case.meta["psi_bcs"].append({"kind": kind, "name": name, "direction": int(direction),
                                         "row": int(row)})
            case.groups["g_" + name] = np.asarray(sorted(map(tuple, group_nodes(ob.group))),
                                                  np.int32).reshape(-1, 2)
    else:
        bsc.add_boundary_condition("periodicBT", tl.PeriodicPsi_BT())
        case.meta["psi_bcs"].append("periodic_bt")
    if fixed_psi is not None:
        row, value = fixed_psi

        @ti.func
        def row_fn(i, j):
            return lb.mask[i, j] == 1 and j == row
        fp = tl.FixedPsi(spec=tl.BoundarySpec(geometry_fn=row_fn), psi_value=value)
        fp.precompute(classifier=cls)
        bsc.add_boundary_condition("fixed", fp)
        case.meta["psi_bcs"].append({"kind": "fixed", "name": "psi_fixed", "value": float(value), "row": int(row)})
        case.groups["g_psi_fixed"] = np.asarray(sorted(map(tuple, group_nodes(fp.group))), np.int32).reshape(-1, 2)

    lb.T.fill(T)
    case.meta["T"] = T
    for (i, j) in group_nodes(fluid.group):
        lb.rho[i, j, 0] = rho_init[i, j]
    lb.init_LBM(coll, fluid.group)
    return lb, me, coll, be, lb.sc_field, bsc


def build_shanchen_mc(ti, tl, case, nx, ny, *, g_coh, rho_init, nu, rho0, T=1.0, gravity=None):
    """Fully periodic multi-component Shan-Chen lattice (ShanChenForceC2,
    SC_psi per component, BGK per component with the mixture velocity): every
    node is fluid, so fluid_strategy is true everywhere and no adhesion acts."""
    nc = len(nu)
    lb = tl.LBField(case.meta["name"], nx, ny, nc)
    if gravity is not None:
        lb.set_gravity(ti.Vector(list(gravity)))
        case.meta["gravity"] = list(gravity)
    be = tl.BoundaryEngine()
    cls = tl.BoundaryClassifier(ti.field(float, shape=(nx, ny)))

    @ti.func
    def fluid_fn(i, j):
        return lb.mask[i, j] == 1
    fluid = tl.FluidBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
    fluid.precompute(classifier=cls)
    be.add_boundary_condition("fluid", fluid)
    case.bc("fluid", "fluid", group_nodes(fluid.group))
    per = tl.PeriodicAllBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
    per.precompute(classifier=cls)
    be.add_boundary_condition("stream", per)
    case.bc("stream", "periodic", group_nodes(per.group))
    lb.neighbor_classify()
    me = tl.MacroscopicEngine(fluid.group)
    params = {"group": fluid.group, "fluid_model": tl.NewtonianFluid(nu[0]), "NX": nx, "NY": ny,
              "num_components": nc, "shearviscosity": list(nu)}
    coll = tl.BGKCollision(params)
    case.meta["collision"] = {"model": "bgk", "nu": list(nu)}

    @ti.func
    def everywhere(i, j):
        return True
    psis = [tl.SC_psi(rho0=r) for r in rho0]
    g = ti.Matrix([list(row) for row in g_coh])
    lb.sc_field = tl.ShanChenForceC2({"lb_field": lb, "g_coh": g, "gadh": [0.0] * nc, "group": fluid.group,
                                      "psi_list": psis, "fluid_strategy": everywhere})
    case.meta["sc"] = {"g_coh": [list(row) for row in g_coh], "psi": [["sc", r] for r in rho0],
                       "components": nc}
    bsc = tl.BoundaryEngineSC()
    bsc.add_boundary_condition("periodicLR", tl.PeriodicPsi_LR())
    bsc.add_boundary_condition("periodicBT", tl.PeriodicPsi_BT())
    case.meta["psi_bcs"] = ["periodic_lr", "periodic_bt"]
    lb.T.fill(T)
    case.meta["T"] = T
    for (i, j) in group_nodes(fluid.group):
        for c in range(nc):
            lb.rho[i, j, c] = rho_init[c][i, j]
    lb.init_LBM(coll, fluid.group)
    return lb, me, coll, be, lb.sc_field, bsc


def build_ibm_box(ti, tl, case, nx, ny, *, center, radius, mdf, nu, gravity):
    """Fully periodic box driven by gravity past one immersed circle (SphereIB
    with IB nodes every unit of arc, IBDEMCouplerEngine placing them, IBEngine
    multi-direct forcing with `mdf` iterations), BGK, the IB step between the
    velocity and the collision (ibm.py)."""
    lb = tl.LBField(case.meta["name"], nx, ny, 1)
    lb.set_gravity(ti.Vector(list(gravity)))
    case.meta["gravity"] = list(gravity)
    be = tl.BoundaryEngine()
    cls = tl.BoundaryClassifier(ti.field(float, shape=(nx, ny)))

    @ti.func
    def fluid_fn(i, j):
        return lb.mask[i, j] == 1
    fluid = tl.FluidBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
    fluid.precompute(classifier=cls)
    be.add_boundary_condition("fluid", fluid)
    case.bc("fluid", "fluid", group_nodes(fluid.group))
    per = tl.PeriodicAllBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
    per.precompute(classifier=cls)
    be.add_boundary_condition("stream", per)
    case.bc("stream", "periodic", group_nodes(per.group))
    lb.neighbor_classify()
    me = tl.MacroscopicEngine(fluid.group)
    coll = make_collision(ti, tl, case, lb, fluid.group, ("bgk", {}), nu, None, None, None)
    sphere = tl.SphereIB(1, 64)
    sphere.init_Balls(1, np.array([0]), np.array([list(center)]), np.array([[0.0, 0.0]]), np.array([[0.0, 0.0]]),
                      np.array([0.0]), np.array([radius]), np.array([0.0]))
    sphere.init_IB_nodes()
    coupler = tl.IBDEMCouplerEngine(lb)
    coupler.SphereInfoUpdata(sphere, np.array([list(center)]), np.array([[0.0, 0.0]]), np.array([0.0]))
    ib = tl.IBEngine(mdf)
    case.meta["ibm"] = {"center": list(center), "radius": radius, "mdf": mdf}
    for (i, j) in group_nodes(fluid.group):
        lb.rho[i, j, 0] = 1.0
    lb.init_LBM(coll, fluid.group)
    return lb, me, coll, be, (sphere, ib), None


def step_fn(lb, me, coll, be, sc, bsc, kind):
    def standard():
        me.density(lb)
        me.pressure(lb)
        me.force_density(lb)
        me.velocity(lb)
        coll.apply(lb)
        be.apply_boundary_conditions(lb)

    def powerlaw():
        me.density(lb)
        me.pressure(lb)
        me.force_density(lb)
        me.velocity(lb)
        coll.shear_rate(lb)
        coll.relaxation_time(lb)
        coll.apply(lb)
        be.apply_boundary_conditions(lb)

    def shanchen():
        me.density(lb)
        me.pressure(lb)
        sc.update_psi(lb)
        bsc.apply_boundary_conditions(lb)
        sc.cau_SCforce(lb)
        me.force_density(lb)
        me.velocity(lb)
        coll.apply(lb)
        be.apply_boundary_conditions(lb)
        me.time_updata(lb)

    def ibm():
        sphere, ib = sc
        me.density(lb)
        me.pressure(lb)
        me.force_density(lb)
        me.velocity(lb)
        ib.MultiDirectForcingLoop(sphere, lb)
        ib.ComputeParticleForce(sphere)
        coll.apply(lb)
        be.apply_boundary_conditions(lb)

    if kind == "ibm":
        def prologue():
            me.density(lb)
            me.pressure(lb)
            me.force_density(lb)
            me.velocity(lb)
        return ibm, prologue

    def prologue():
        me.density(lb)
        me.pressure(lb)
        if sc is not None:
            sc.update_psi(lb)
            bsc.apply_boundary_conditions(lb)
            sc.cau_SCforce(lb)
        me.force_density(lb)
        me.velocity(lb)

    return {"standard": standard, "powerlaw": powerlaw, "shanchen": shanchen}[kind], prologue


def cs_params(T_over_Tc):
    a, b, R = 1.0, 4.0, 1.0
    Tc = 0.3773 * a / (b * R)
    return {"a": a, "b": b, "R": R, "G": -1.0, "rho_cr": 0.1304 / b * 4.0,
            "pressure_cr": 0.0707 * a / b ** 2, "temperature_cr": Tc}, T_over_Tc * Tc


def powerlaw_K(umax, L, n, Re):
    return umax ** (2.0 - n) * L ** n / Re


def case_table():
    """name -> (builder kwargs, step kind, steps)."""
    nx, ny = 40, 20
    cyl = dict(disc=(10.0, 9.5, 3.5), stream="periodic", inlet=("eq_parabolic", 0.05),
               outlet=("pressure_neem", 1.0), nu=0.02)
    ll = lambda tau: (0.0, 1.64, 1.54, 0.0, 1.7, 0.0, 1.7, 1.0 / tau, 1.0 / tau)  # noqa: E731
    t = {}
    t["cyl_bgk_f32"] = ("channel", dict(cyl, collision=("bgk", {})), "standard", 40, "f32", (nx, ny))
    t["cyl_bgk_f64"] = ("channel", dict(cyl, collision=("bgk", {})), "standard", 40, "f64", (nx, ny))
    t["cyl_trt_f32"] = ("channel", dict(cyl, collision=("trt", {"magic": [0.25]})), "standard", 40,
                        "f32", (nx, ny))
    t["cyl_mrt_f32"] = ("channel", dict(cyl, collision=("mrt", {"bulkviscosity": [0.05]})),
                        "standard", 30, "f32", (nx, ny))
    t["cyl_mrt_ll_f32"] = ("channel", dict(cyl, collision=("mrt", {"bulkviscosity": [0.05]}),
                                           mrt_diag=ll(0.56)), "standard", 30, "f32", (nx, ny))
    t["chan_inside_eq_bgk_f32"] = ("channel", dict(disc=(12.0, 7.0, 2.5), stream="inside",
                                                   inlet=("eq", 0.04), outlet=("pressure_neem", 1.0),
                                                   collision=("bgk", {}), nu=0.03),
                                   "standard", 40, "f32", (32, 16))
    t["chan_vneem_neumann_trt_f32"] = ("channel", dict(stream="periodic", inlet=("neem", 0.03),
                                                       outlet=("open_neumann", None),
                                                       collision=("trt", {"magic": [0.1875]}),
                                                       nu=0.04), "standard", 40, "f32", (32, 16))
    t["chan_vbb_abc_bgk_f32"] = ("channel", dict(stream="periodic", inlet=("bb", 0.03),
                                                 outlet=("pressure_abc", 1.0),
                                                 collision=("bgk", {}), nu=0.05),
                                 "standard", 40, "f32", (32, 16))
    t["chan_eq_conv1_bgk_f32"] = ("channel", dict(disc=(10.0, 8.0, 2.5), stream="periodic",
                                                  inlet=("eq", 0.03), outlet=("open_conv1", None),
                                                  collision=("bgk", {}), nu=0.04),
                                  "standard", 40, "f32", (32, 16))
    t["chan_eq_extrap_mrt_f32"] = ("channel", dict(stream="periodic", inlet=("eq", 0.03),
                                                   outlet=("open_extrap", None),
                                                   collision=("mrt", {"bulkviscosity": [0.04]}),
                                                   nu=0.04), "standard", 30, "f32", (32, 16))
    t["pois_gravity_bgk_f32"] = ("channel", dict(stream="periodic", inlet=("eq", 0.0),
                                                 outlet=("pressure_neem", 1.0),
                                                 collision=("bgk", {}), nu=0.1,
                                                 gravity=(1e-5, 0.0)), "standard", 40, "f32", (24, 12))
    # power-law 4:1-style contraction: outlet section of height 8 for x >= 24
    cnx, cny, h, x0 = 48, 24, 8, 24
    rects = ((x0 - 0.5, cnx + 0.5, -0.5, (cny - h) / 2 - 0.5),
             (x0 - 0.5, cnx + 0.5, (cny + h) / 2 - 0.5, cny + 0.5))
    for n, model in ((0.5, "trt"), (1.5, "trt"), (1.0, "trt"), (1.5, "bgk"), (0.5, "mrt")):
        K = powerlaw_K(0.02, cny, n, 20.0)
        extra = {"trt": {"magic": [0.25]}, "bgk": {}, "mrt": {"bulkviscosity": [K]}}[model]
        name = f"contraction_pl_{model}_n{str(n).replace('.', '')}_f32"
        t[name] = ("channel", dict(rects=rects, stream="periodic", inlet=("eq_parabolic", 0.02),
                                   outlet=("pressure_neem", 1.0), collision=(model, extra), nu=K,
                                   fluid_model=(K, n), tau_clamp=(0.505, 2.0)),
                   "powerlaw", 30, "f32", (cnx, cny))
    rng = np.random.Generator(np.random.PCG64(SEED))
    p, T = cs_params(0.8)
    rho_cs = (0.25 * (1.0 + rng.uniform(-0.01, 0.01, size=(24, 20)))).astype(np.float64)
    t["sc_cs_bgk_f32"] = ("shanchen", dict(eos=("cs", p), g_coh=-1.0, rho_init=rho_cs,
                                           collision=("bgk", {}), nu=0.5 / 3.0, T=T),
                          "shanchen", 40, "f32", (24, 20))
    rho_sc = (np.log(2.0) + 0.1 * rng.uniform(0.0, 1.0, size=(20, 18))).astype(np.float64)
    t["sc_scpsi_mrt_f32"] = ("shanchen", dict(eos=("sc", 1.0), g_coh=-5.0, rho_init=rho_sc,
                                              collision=("mrt", {"bulkviscosity": [0.1]}),
                                              nu=0.1, T=1.0, gravity=(0.0, -1e-5)),
                             "shanchen", 30, "f32", (20, 18))
    rho_vdw = (0.3 * (1.0 + rng.uniform(-0.02, 0.02, size=(16, 16)))).astype(np.float64)
    t["sc_vdw_trt_f64"] = ("shanchen", dict(eos=("vdw", {"a": 9.0 / 49.0, "b": 2.0 / 21.0, "R": 1.0,
                                                         "G": -1.0, "rho_cr": 3.5,
                                                         "pressure_cr": 0.0, "temperature_cr": 4.0 / 7.0}),
                                            g_coh=-1.0, rho_init=rho_vdw,
                                            collision=("trt", {"magic": [0.25]}), nu=0.1,
                                            T=0.85 * 4.0 / 7.0), "shanchen", 30, "f64", (16, 16))
    # Redlich-Kwong and Peng-Robinson pseudopotentials (EOS.py:61-83), the
    # Yuan-Schaefer parameters a = 2/49, b = 2/21, R = 1, near their critical
    # densities at T = 0.9 Tc.  These cases draw from their own generator, so
    # the inputs of the cases after them stay as they were.
    rng2 = np.random.Generator(np.random.PCG64(SEED + 1))
    rk = {"a": 2.0 / 49.0, "b": 2.0 / 21.0, "R": 1.0, "G": -1.0, "rho_cr": 2.729,
          "pressure_cr": 0.1779, "temperature_cr": 0.1961}
    rho_rk = (2.6 * (1.0 + rng2.uniform(-0.01, 0.01, size=(24, 20)))).astype(np.float64)
    t["sc_rk_bgk_f32"] = ("shanchen", dict(eos=("rk", rk), g_coh=-1.0, rho_init=rho_rk,
                                           collision=("bgk", {}), nu=0.5 / 3.0, T=0.9 * 0.1961),
                          "shanchen", 30, "f32", (24, 20))
    pr = {"a": 2.0 / 49.0, "b": 2.0 / 21.0, "R": 1.0, "G": -1.0, "rho_cr": 2.657,
          "pressure_cr": 0.0585, "temperature_cr": 0.0729, "omega": 0.344}
    rho_pr = (2.5 * (1.0 + rng2.uniform(-0.01, 0.01, size=(20, 16)))).astype(np.float64)
    t["sc_pr_trt_f32"] = ("shanchen", dict(eos=("pr", pr), g_coh=-1.0, rho_init=rho_pr,
                                           collision=("trt", {"magic": [0.25]}), nu=0.1, T=0.9 * 0.0729),
                          "shanchen", 30, "f32", (20, 16))
    # FixedPsi (SCBoundaryCondition.py:113-123) on the bottom row, after the
    # periodic psi boundaries
    rho_fx = (np.log(2.0) + 0.1 * rng2.uniform(0.0, 1.0, size=(20, 18))).astype(np.float64)
    t["sc_fixedpsi_bgk_f32"] = ("shanchen", dict(eos=("sc", 1.0), g_coh=-5.0, rho_init=rho_fx,
                                                 collision=("bgk", {}), nu=0.1, T=1.0, fixed_psi=(0, 0.3)),
                                "shanchen", 30, "f32", (20, 18))
    # OpenConvective2order (BoundaryCondition.py:362-390) on the last column
    # of a Shan-Chen lattice, after the periodic stream
    rho_oc = (0.25 * (1.0 + rng2.uniform(-0.01, 0.01, size=(24, 20)))).astype(np.float64)
    p_oc, T_oc = cs_params(0.85)
    t["sc_openconv2_bgk_f32"] = ("shanchen", dict(eos=("cs", p_oc), g_coh=-1.0, rho_init=rho_oc,
                                                  collision=("bgk", {}), nu=0.5 / 3.0, T=T_oc, open_conv2=True),
                                 "shanchen", 30, "f32", (24, 20))
    # the open psi boundaries (SCBoundaryCondition.py:19-110) on the halo rows
    # below and above the lattice (psi periodic in x)
    rho_op = (0.25 * (1.0 + rng2.uniform(-0.01, 0.01, size=(24, 20)))).astype(np.float64)
    p_op, T_op = cs_params(0.8)
    t["sc_openpsi_bgk_f32"] = ("shanchen", dict(eos=("cs", p_op), g_coh=-1.0, rho_init=rho_op,
                                                collision=("bgk", {}), nu=0.5 / 3.0, T=T_op,
                                                open_psi=[("open_neumann_psi", 20, 2),
                                                          ("open_extrap_psi", -1, 4)]),
                               "shanchen", 30, "f32", (24, 20))
    t["sc_openpsiconv_trt_f32"] = ("shanchen", dict(eos=("cs", p_op), g_coh=-1.0, rho_init=rho_op,
                                                    collision=("trt", {"magic": [0.25]}), nu=0.1, T=T_op,
                                                    gravity=(1e-5, 0.0),
                                                    open_psi=[("open_conv1_psi", 20, 2),
                                                              ("open_conv2_psi", -1, 4)]),
                                   "shanchen", 30, "f32", (24, 20))
    # two components: a disc of component 0 in component 1, seeded noise
    mx, my = 24, 20
    ii, jj = np.meshgrid(np.arange(mx), np.arange(my), indexing="ij")
    disc = ((ii - 11.5) ** 2 + (jj - 9.5) ** 2) < 36.0
    a = np.where(disc, 1.0, 0.06) * (1.0 + rng.uniform(-0.01, 0.01, size=(mx, my)))
    b = np.where(disc, 0.06, 1.0) * (1.0 + rng.uniform(-0.01, 0.01, size=(mx, my)))
    for fp in ("f32", "f64"):
        t[f"mc_sc2_bgk_{fp}"] = ("shanchen_mc", dict(g_coh=((0.0, 0.9), (0.9, 0.0)), rho_init=(a, b),
                                                    nu=(1.0 / 6.0, 0.1), rho0=(1.0, 1.0),
                                                    gravity=(0.0, -1e-5) if fp == "f32" else None),
                                 "shanchen", 30, fp, (mx, my))
    t["ibm_circle_bgk_f32"] = ("ibm", dict(center=(16.0, 12.0), radius=4.0, mdf=2, nu=0.1,
                                           gravity=(1e-5, 0.0)), "ibm", 30, "f32", (32, 24))
    return t


def run_case(ref_root, name, spec, out_dir):
    builder, kw, kind, steps, fp, (nx, ny) = spec
    ti, tl = load_reference(ref_root, fp)
    case = Case(name, nx, ny, fp)
    case.meta["steps"] = steps
    case.meta["step_kind"] = kind
    t0 = time.time()
    with contextlib.redirect_stdout(io.StringIO()), warnings.catch_warnings():
        warnings.simplefilter("ignore")
        if builder == "channel":
            lb, me, coll, be, sc, bsc = build_channel(ti, tl, case, nx, ny, **kw)
        elif builder == "shanchen_mc":
            lb, me, coll, be, sc, bsc = build_shanchen_mc(ti, tl, case, nx, ny, **kw)
        elif builder == "ibm":
            lb, me, coll, be, sc, bsc = build_ibm_box(ti, tl, case, nx, ny, **kw)
        else:
            lb, me, coll, be, sc, bsc = build_shanchen(ti, tl, case, nx, ny, **kw)
        init_rho_all = lb.rho.to_numpy().copy()
        init_rho = lb.rho.to_numpy()[:, :, 0].copy()
        init_vel = lb.vel.to_numpy().copy()
        step, prologue = step_fn(lb, me, coll, be, sc, bsc, kind)
        for _ in range(steps):
            step()
        prologue()
    out = dict(case.groups)
    out["mask"] = lb.mask.to_numpy()
    out["neighbor"] = lb.neighbor.to_numpy()
    out["init_rho"] = init_rho
    out["init_vel"] = init_vel
    out["f"] = lb.f.to_numpy()[:, :, 0, :]
    out["f2"] = lb.f2.to_numpy()[:, :, 0, :]
    out["rho"] = lb.rho.to_numpy()[:, :, 0]
    out["total_rho"] = lb.total_rho.to_numpy()
    out["vel"] = lb.vel.to_numpy()
    out["body_force"] = lb.body_force.to_numpy()[:, :, 0, :]
    out["pressure"] = lb.total_pressure.to_numpy()
    out["shear_rate"] = lb.shear_rate.to_numpy()[:, :, 0]
    model = case.meta["collision"]["model"]
    if model == "bgk":
        out["tau"] = coll.tau.to_numpy()[:, :, 0]
    elif model == "trt":
        out["tau_sym"] = coll.tau_sym.to_numpy()[:, :, 0]
        out["tau_antisym"] = coll.tau_antisym.to_numpy()[:, :, 0]
    else:
        out["diag"] = coll.diag.to_numpy()[:, :, 0, :]
        out["M_inverse"] = coll.M_inverse.to_numpy()
    if builder == "ibm":  # the immersed circle's nodes and the resultant
        sphere, _ = sc
        for k in ("pos", "vel", "vel_desired", "force", "force_temp"):
            out["ib_" + k] = getattr(sphere.IBNodes, k).to_numpy()[0, :sphere.Sphere[0].NumIB]
        out["ib_count"] = np.array(sphere.IBInsiderCount[None])
        out["sphere_force"] = sphere.Sphere.force.to_numpy()[0]
        out["sphere_torque"] = np.array(sphere.Sphere.torque.to_numpy()[0])
        sc = None
    if sc is not None:
        out["psi"] = sc.psi_field.to_numpy()[:, :, 0]
        out["sc_force"] = lb.SCforce.to_numpy()[:, :, 0, :]
        out["T"] = lb.T.to_numpy()
    if builder == "shanchen_mc":  # every component, [i, j, component, ...]
        out["init_rho_mc"] = init_rho_all
        out["f_mc"] = lb.f.to_numpy()
        out["f2_mc"] = lb.f2.to_numpy()
        out["rho_mc"] = lb.rho.to_numpy()
        out["psi_mc"] = sc.psi_field.to_numpy()
        out["sc_force_mc"] = lb.SCforce.to_numpy()
        out["body_force_mc"] = lb.body_force.to_numpy()
        out["pressure_mc"] = lb.pressure.to_numpy()
    out["meta"] = np.array(json.dumps(case.meta))
    np.savez_compressed(os.path.join(out_dir, name + ".npz"), **out)
    return time.time() - t0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("TAICHI_LBM_REF"),
                    help="checkout of the reference (default: $TAICHI_LBM_REF)")
    ap.add_argument("--out", default=HERE)
    ap.add_argument("cases", nargs="*")
    a = ap.parse_args()
    if not a.ref:
        raise SystemExit("give the reference checkout with --ref PATH or TAICHI_LBM_REF")
    table = case_table()
    names = a.cases or list(table)
    for n in names:
        # one process per case: the Taichi stand-in's default float type is global
        if len(names) > 1:
            rc = os.spawnv(os.P_WAIT, sys.executable,
                           [sys.executable, __file__, "--ref", a.ref, "--out", a.out, n])
            if rc != 0:
                raise SystemExit(f"case {n} failed ({rc})")
            continue
        dt = run_case(a.ref, n, table[n], a.out)
        print(f"{n}: {dt:.1f}s", flush=True)


if __name__ == "__main__":
    main()
