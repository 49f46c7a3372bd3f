"""GPU parity of the immersed-boundary coupling (taichi_lbm.ibm: SphereIB,
IBDEMCouplerEngine, IBEngine over lbm_ibm_interpolate / lbm_ibm_spread)
against the reference fixture tests/golden/ibm_circle_bgk_f32.npz (a circle
of IB nodes in a gravity-driven periodic box, two multi-direct forcing
iterations between the velocity and the BGK collision, 30 steps), the case
oracle/ibm.py reproduces bit for bit.  The spread adds atomically, so sums
into a grid node shared by several IB nodes may round in another order:
bound 1e-5 of each field's maximum.
"""
import json

import numpy as np
import pytest

from tests.cases import ROOT, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def build(tl, meta, arrays):
    nx, ny = meta["NX"], meta["NY"]
    lb = tl.LBField("ibm", nx, ny, 1)
    lb.set_gravity(list(meta["gravity"]))
    cls = tl.BoundaryClassifier((nx, ny))
    be = tl.BoundaryEngine()
    fl = tl.FluidBoundary(spec=tl.BoundarySpec(geometry_fn=lambda i, j: lb.mask[i, j] == 1))
    fl.precompute(cls)
    be.add_boundary_condition("fluid", fl)
    per = tl.PeriodicAllBoundary(spec=tl.BoundarySpec(geometry_fn=lambda i, j: lb.mask[i, j] == 1))
    per.precompute(cls)
    be.add_boundary_condition("stream", per)
    lb.neighbor_classify()
    me = tl.MacroscopicEngine(fl.group)
    nu = meta["collision"]["nu"][0]
    coll = tl.BGKCollision({"group": fl.group, "fluid_model": tl.NewtonianFluid(nu), "NX": nx, "NY": ny,
                            "num_components": 1, "shearviscosity": [nu]})
    ib = meta["ibm"]
    sphere = tl.SphereIB(1, 64)
    c = np.array([ib["center"]])
    sphere.init_Balls(1, np.array([0]), c, np.zeros((1, 2)), np.zeros((1, 2)), np.zeros(1),
                      np.array([ib["radius"]]), np.zeros(1))
    sphere.init_IB_nodes()
    coupler = tl.IBDEMCouplerEngine(lb)
    coupler.SphereInfoUpdata(sphere, c, np.zeros((1, 2)), np.zeros(1))
    engine = tl.IBEngine(ib["mdf"])
    lb.rho.from_numpy(np.asarray(arrays["init_rho"], np.float32)[:, :, None])
    lb.vel.fill([0.0, 0.0])
    lb.init_LBM(coll, fl.group)
    return lb, me, coll, be, sphere, engine


def test_immersed_circle_matches_reference(tl):
    d = np.load(f"{ROOT}/tests/golden/ibm_circle_bgk_f32.npz")
    meta = json.loads(str(d["meta"]))
    arrays = {k: d[k] for k in d.files if k != "meta"}
    lb, me, coll, be, sphere, engine = build(tl, meta, arrays)
    assert sphere.IBInsiderCount[None] == int(arrays["ib_count"])
    for _ in range(meta["steps"]):
        me.density(lb)
        me.pressure(lb)
        me.force_density(lb)
        me.velocity(lb)
        engine.MultiDirectForcingLoop(sphere, lb)
        engine.ComputeParticleForce(sphere)
        coll.apply(lb)
        be.apply_boundary_conditions(lb)
    me.density(lb)
    me.pressure(lb)
    me.force_density(lb)
    me.velocity(lb)
    n = sphere.Sphere.NumIB[0]
    got = {"f": lb.f.to_numpy()[:, :, 0, :], "rho": lb.rho.to_numpy()[:, :, 0], "vel": lb.vel.to_numpy(),
           "body_force": lb.body_force.to_numpy()[:, :, 0, :],
           "ib_pos": sphere.IBNodes.pos.to_numpy()[0, :n], "ib_vel": sphere.IBNodes.vel.to_numpy()[0, :n],
           "ib_force": sphere.IBNodes.force.to_numpy()[0, :n],
           "sphere_force": sphere.Sphere.force.to_numpy()[0]}
    for k, v in got.items():
        assert rel_err(v, arrays[k]) <= 1e-5, (k, rel_err(v, arrays[k]))
