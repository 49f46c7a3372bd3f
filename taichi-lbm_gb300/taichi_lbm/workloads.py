"""Benchmark workloads built through the drop-in API.

cylinder_channel: the reference's cylinder case (cases/Circular cylinder.py)
as a channel with walls on every lattice edge, with boundary groups that
never index outside the lattice, and a parabolic inlet given per node through
BoundarySpec.value_fn.
"""
import numpy as np


def cylinder_channel(tl, nx, ny, radius, cx, cy, tau, umax, model="bgk", mrt_s=None, magic=0.25,
                     name="cylinder", keep_init=True):
    """Channel with a cylinder: walls on every lattice edge (bounce-back for
    every missing link), periodic stream carrier, parabolic VelocityEquilibrium
    inlet at i = 0 (direction 3), PressureNEEM outlet rho = 1 at i = NX-1
    (direction 1) — the reference's cylinder case with out-of-range-free groups."""
    lb = tl.LBField(name, nx, ny, 1)
    lb.keep_init_snapshot = keep_init
    be = tl.BoundaryEngine()
    be.Mask_cricle_identify(lb, cx, cy, radius)
    cls = tl.BoundaryClassifier((nx, ny))
    mask = lb.mask.arr

    def fluid_fn(i, j):
        return mask[i, j] == 1

    def missing_link(i, j):
        flag = np.zeros(np.shape(i), bool)
        for k in range(9):
            i2, j2 = i - lb.c[k, 0], j - lb.c[k, 1]
            out = (i2 < 0) | (i2 > nx - 1) | (j2 < 0) | (j2 > ny - 1)
            solid = np.zeros(np.shape(i), bool)
            ok = ~out
            solid[ok] = mask[i2[ok], j2[ok]] == -1
            flag |= out | solid
        return flag

    def wall_fn(i, j):
        return (mask[i, j] == 1) & missing_link(i, j)

    def inlet_fn(i, j):
        return (mask[i, j] == 1) & (i == 0)

    def outlet_fn(i, j):
        return (mask[i, j] == 1) & (i == nx - 1)

    def parabola(i, j):
        y = j + 0.5
        return (4.0 * umax * y * (ny - y) / (ny * ny), np.zeros(np.shape(j)))

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
    params = {"group": fluid.group, "fluid_model": tl.NewtonianFluid(nu=nu), "NX": nx, "NY": ny,
              "num_components": 1, "shearviscosity": [nu], "magic": [magic], "bulkviscosity": [nu]}
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
