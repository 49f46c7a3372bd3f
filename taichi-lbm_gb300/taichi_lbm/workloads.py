"""Benchmark workloads built through the drop-in API.

cylinder_channel: the reference's cylinder case (cases/Circular cylinder.py)
as a channel with walls on every lattice edge, with boundary groups that
never index outside the lattice, and a parabolic inlet given per node through
BoundarySpec.value_fn.  contraction_channel: the planar contraction of
cases/contraction flow.py with a power-law fluid.
"""
import numpy as np


def cylinder_channel(tl, nx, ny, radius, cx, cy, tau, umax, model="bgk", mrt_s=None, magic=0.25,
                     name="cylinder", keep_init=True, powerlaw=None, tau_clamp=None):
    """Channel with a cylinder: walls on every lattice edge (bounce-back for
    every missing link), periodic stream carrier, parabolic VelocityEquilibrium
    inlet at i = 0 (direction 3), PressureNEEM outlet rho = 1 at i = NX-1
    (direction 1) — the reference's cylinder case with out-of-range-free groups.
    powerlaw=(m, n) makes the fluid a PowerLawFluid (local relaxation)."""
    lb = tl.LBField(name, nx, ny, 1)
    lb.keep_init_snapshot = keep_init
    be = tl.BoundaryEngine()
    be.Mask_cricle_identify(lb, cx, cy, radius)
    return _channel(tl, lb, be, nx, ny, tau, umax, 0, ny, model, mrt_s, magic, powerlaw, tau_clamp)


def contraction_channel(tl, nx=2048, ny=512, outlet_h=128, n=1.0, re=20.0, umax=0.02, model="trt",
                        tau_clamp=(0.505, 2.0), magic=0.25, name="contraction", keep_init=False):
    """Planar contraction (the reference's cases/contraction flow.py, scaled):
    a channel of height NY whose second half (x >= NX/2) is closed above and
    below by solid, leaving an outlet section `outlet_h` high in the middle
    (two Mask_rectangle_identify rectangles).  Parabolic inlet of peak `umax`
    over the full height, PressureNEEM outlet, bounce-back walls, power-law
    fluid of index n with the consistency m of Reynolds number `re` on the
    outlet height (m = umax^(2-n) outlet_h^n / Re, as cases/Power Law
    Fluid.py:41 relates K to Re), relaxation time clamped to `tau_clamp`.
    The initial tau is that of the nominal shear rate umax / outlet_h."""
    lb = tl.LBField(name, nx, ny, 1)
    lb.keep_init_snapshot = keep_init
    be = tl.BoundaryEngine()
    lo, hi = (ny - outlet_h) // 2, (ny + outlet_h) // 2
    # open rectangles: x in (nx/2 - 1, nx + 1), y in (-1, lo) and (hi - 1, ny + 1)
    be.Mask_rectangle_identify(lb, nx // 2 - 1, nx + 1, -1, lo)
    be.Mask_rectangle_identify(lb, nx // 2 - 1, nx + 1, hi - 1, ny + 1)
    m = umax ** (2.0 - n) * float(outlet_h) ** n / re
    nu0 = m * (umax / outlet_h) ** (n - 1.0)
    tau = min(max(0.5 + 3.0 * nu0, tau_clamp[0]), tau_clamp[1])
    return _channel(tl, lb, be, nx, ny, tau, umax, 0, ny, model, None, magic, (m, n), tau_clamp)


def _channel(tl, lb, be, nx, ny, tau, umax, y0, y1, model, mrt_s, magic, powerlaw, tau_clamp):
    """Boundary groups and collision of a channel whose solid is already in
    lb.mask: bounce-back for every missing link, periodic carrier, parabolic
    inlet over rows [y0, y1) at i = 0, PressureNEEM outlet at i = NX-1."""
    cls = tl.BoundaryClassifier((nx, ny))
    mask = lb.mask.arr
    fluid_arr = mask == 1
    # a fluid node is a wall node when one of its links has its source outside
    # the lattice or in the solid
    src_ok = np.pad(mask != -1, 1, constant_values=False)
    missing = np.zeros((nx, ny), bool)
    for k in range(9):
        ex, ey = int(lb.c[k, 0]), int(lb.c[k, 1])
        missing |= ~src_ok[1 - ex:1 - ex + nx, 1 - ey:1 - ey + ny]
    wall_arr = fluid_arr & missing
    h = float(y1 - y0)

    def fluid_fn(i, j):
        return fluid_arr[i, j]

    def wall_fn(i, j):
        return wall_arr[i, j]

    def inlet_fn(i, j):
        return fluid_arr[i, j] & (i == 0)

    def outlet_fn(i, j):
        return fluid_arr[i, j] & (i == nx - 1)

    def parabola(i, j):
        y = np.clip(j + 0.5 - y0, 0.0, h)
        return (4.0 * umax * y * (h - y) / (h * h), np.zeros(np.shape(j)))

    fluid = tl.FluidBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
    fluid.precompute(classifier=cls)
    be.add_boundary_condition("fluid", fluid)
    per = tl.PeriodicAllBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
    per.precompute(classifier=cls)
    be.add_boundary_condition("periodic", per)
    wall = tl.BounceBackWall(spec=tl.BoundarySpec(geometry_fn=wall_fn))
    wall.precompute(classifier=cls)
    be.add_boundary_condition("wall", wall)
    inlet = tl.VelocityEquilibrium(spec=tl.BoundarySpec(geometry_fn=inlet_fn, value_fn=parabola),
                                   velocity_value=[umax, 0.0], direction=3)
    inlet.precompute(classifier=cls)
    be.add_boundary_condition("inlet", inlet)
    outlet = tl.PressureNEEM(spec=tl.BoundarySpec(geometry_fn=outlet_fn), rho_value=1.0, direction=1)
    outlet.precompute(classifier=cls)
    be.add_boundary_condition("outlet", outlet)
    lb.neighbor_classify()
    me = tl.MacroscopicEngine(fluid.group)
    nu = (tau - 0.5) / 3.0
    fluid_model = tl.NewtonianFluid(nu=nu) if powerlaw is None else tl.PowerLawFluid(*powerlaw)
    params = {"group": fluid.group, "fluid_model": fluid_model, "NX": nx, "NY": ny,
              "num_components": 1, "shearviscosity": [nu], "magic": [magic], "bulkviscosity": [nu]}
    if tau_clamp is not None:
        params["tau_clamp"] = tau_clamp
    if model == "bgk":
        coll = tl.BGKCollision(params)
    elif model == "trt":
        coll = tl.TRTCollision(params)
    else:
        if mrt_s is not None:
            params["mrt_s"] = mrt_s
        coll = tl.MRTCollision(params)
    lb.rho.fill(0.0)
    nd = fluid.group.nodes
    rho0 = np.zeros((nx, ny, 1), np.float32)
    rho0[nd[:, 0], nd[:, 1]] = 1.0
    lb.rho.from_numpy(rho0)
    lb.vel.fill([0.0, 0.0])
    lb.init_LBM(coll, fluid.group)
    return lb, me, coll, be


def carnahan_starling(tl, T_over_Tc, a=1.0, b=4.0, R=1.0, G=-1.0):
    """CS_psi with a, b, R and the temperature T = (T/Tc) Tc, Tc = 0.3773 a / (b R)."""
    Tc = 0.3773 * a / (b * R)
    psi = tl.CS_psi({"a": a, "b": b, "R": R, "G": G, "rho_cr": 0.1304 / b * 4.0,
                     "pressure_cr": 0.0707 * a / b ** 2, "temperature_cr": Tc})
    return psi, T_over_Tc * Tc


def shan_chen_box(tl, nx, ny, psi, g_coh, T, rho_init, model="bgk", tau=1.0, magic=0.25,
                  name="shan_chen", keep_init=True):
    """Fully periodic single-component Shan-Chen lattice (the reference's
    two-phase separation case, cases/Bubble or two-phase separation.py):
    periodic stream carrier, PeriodicPsi_LR + PeriodicPsi_BT, uniform T,
    initial density rho_init (NX, NY), u = 0."""
    lb = tl.LBField(name, nx, ny, 1)
    lb.keep_init_snapshot = keep_init
    be = tl.BoundaryEngine()
    cls = tl.BoundaryClassifier((nx, ny))
    mask = lb.mask.arr

    def fluid_fn(i, j):
        return mask[i, j] == 1

    fluid = tl.FluidBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
    fluid.precompute(classifier=cls)
    be.add_boundary_condition("fluid", fluid)
    per = tl.PeriodicAllBoundary(spec=tl.BoundarySpec(geometry_fn=fluid_fn))
    per.precompute(classifier=cls)
    be.add_boundary_condition("stream", per)
    lb.neighbor_classify()
    me = tl.MacroscopicEngine(fluid.group)
    nu = (tau - 0.5) / 3.0
    params = {"group": fluid.group, "fluid_model": tl.NewtonianFluid(nu=nu), "NX": nx, "NY": ny,
              "num_components": 1, "shearviscosity": [nu], "magic": [magic], "bulkviscosity": [nu]}
    coll = {"bgk": tl.BGKCollision, "trt": tl.TRTCollision, "mrt": tl.MRTCollision}[model](params)
    sc = tl.ShanChenForceC1({"lb_field": lb, "g_coh": g_coh, "group": fluid.group, "psi": psi})
    lb.sc_field = sc
    bsc = tl.BoundaryEngineSC()
    bsc.add_boundary_condition("periodicLR", tl.PeriodicPsi_LR())
    bsc.add_boundary_condition("periodicBT", tl.PeriodicPsi_BT())
    lb.T.fill(float(T))
    lb.rho.from_numpy(np.asarray(rho_init, np.float32).reshape(nx, ny, 1))
    lb.vel.fill([0.0, 0.0])
    lb.init_LBM(coll, fluid.group)
    return lb, me, coll, be, sc, bsc


def batched_shan_chen(tl, count=64, sides=tuple(range(128, 1025, 64)), seed=20261203, tt_range=(0.7, 0.9),
                      g_coh=-1.0, tau=1.0, model="bgk", keep_init=False):
    """Many independent periodic Shan-Chen lattices of uneven sizes: side L
    drawn uniformly from `sides`, Carnahan-Starling EOS (a=1, b=4, R=1) at
    T/Tc ~ U[tt_range], rho0 = 0.25 (1 + U[-0.01, 0.01]), all from one seeded
    numpy PCG64 generator.  Returns a list of (lb, me, coll, be, sc, bsc)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = rng.choice(np.asarray(sides), size=count)
    tt = rng.uniform(tt_range[0], tt_range[1], size=count)
    out = []
    for n in range(count):
        side = int(L[n])
        psi, T = carnahan_starling(tl, float(tt[n]))
        rho0 = 0.25 * (1.0 + rng.uniform(-0.01, 0.01, size=(side, side)))
        out.append(shan_chen_box(tl, side, side, psi, g_coh, T, rho0, model=model, tau=tau,
                                 name=f"sc{n}", keep_init=keep_init))
    return out
