"""Two-component Shan-Chen on the GPU (LBField with num_components = 2,
ShanChenForceC2, MacroscopicEngine.pressure2, BGKCollision per component with
the mixture velocity, PeriodicPsi_LR/BT and PeriodicAllBoundary on every
component) against the reference's own source: the fixtures
tests/golden/mc_sc2_bgk_{f32,f64}.npz, which oracle/multicomponent.py
reproduces (tests/test_oracle_multicomponent.py).  The step is the one the
reference's example driver composes (cases/Bubble or two-phase
separation.py:197-212), through the drop-in API, per-stage kernels.

Bound: every field within 1e-5 of its maximum against the f32 fixture (the
fixture's own stand-in sums some products in another order, 2e-6 apart from
the oracle), and within 1e-5 against the f64 one (the fp32 run's rounding
over 30 steps)."""
import json

import numpy as np
import pytest

from tests.cases import ROOT, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def load(name):
    d = np.load(f"{ROOT}/tests/golden/{name}.npz")
    return json.loads(str(d["meta"])), {k: d[k] for k in d.files if k != "meta"}


def build(tl, meta, arrays):
    nx, ny = meta["NX"], meta["NY"]
    sc = meta["sc"]
    nc = int(sc["components"])
    lb = tl.LBField("mc", nx, ny, nc)
    if any(meta.get("gravity", [0.0, 0.0])):
        lb.set_gravity(meta["gravity"])
    cls = tl.BoundaryClassifier((nx, ny))
    be = tl.BoundaryEngine()
    fluid = tl.FluidBoundary(spec=tl.BoundarySpec(geometry_fn=lambda i, j: lb.mask[i, j] == 1))
    fluid.precompute(cls)
    be.add_boundary_condition("fluid", fluid)
    per = tl.PeriodicAllBoundary(spec=tl.BoundarySpec(geometry_fn=lambda i, j: lb.mask[i, j] == 1))
    per.precompute(cls)
    be.add_boundary_condition("stream", per)
    lb.neighbor_classify()
    me = tl.MacroscopicEngine(fluid.group)
    nu = meta["collision"]["nu"]
    coll = tl.BGKCollision({"group": fluid.group, "fluid_model": tl.NewtonianFluid(nu[0]), "NX": nx, "NY": ny,
                            "num_components": nc, "shearviscosity": nu})
    psis = [tl.SC_psi(rho0=p[1]) for p in sc["psi"]]
    lb.sc_field = tl.ShanChenForceC2({"lb_field": lb, "g_coh": sc["g_coh"], "gadh": [0.0] * nc,
                                      "group": fluid.group, "psi_list": psis,
                                      "fluid_strategy": lambda i, j: True})
    bsc = tl.BoundaryEngineSC()
    bsc.add_boundary_condition("periodicLR", tl.PeriodicPsi_LR())
    bsc.add_boundary_condition("periodicBT", tl.PeriodicPsi_BT())
    lb.T.fill(meta.get("T", 1.0))
    lb.rho.from_numpy(np.asarray(arrays["init_rho_mc"], np.float32))
    lb.vel.fill([0.0, 0.0])
    lb.init_LBM(coll, fluid.group)
    return lb, me, coll, be, bsc


def run(tl, meta, arrays):
    lb, me, coll, be, bsc = build(tl, meta, arrays)
    sc = lb.sc_field

    def moments():
        me.density(lb)
        me.pressure(lb)
        sc.update_psi(lb)
        bsc.apply_boundary_conditions(lb)
        sc.cau_SCforce(lb)
        me.force_density(lb)
        me.velocity(lb)

    for _ in range(meta["steps"]):
        moments()
        coll.apply(lb)
        be.apply_boundary_conditions(lb)
        me.time_updata(lb)
    moments()
    return {"f_mc": lb.f.to_numpy(), "f2_mc": lb.f2.to_numpy(), "rho_mc": lb.rho.to_numpy(),
            "total_rho": lb.total_rho.to_numpy(), "vel": lb.vel.to_numpy(), "psi_mc": sc.psi_field.to_numpy(),
            "sc_force_mc": lb.SCforce.to_numpy(), "body_force_mc": lb.body_force.to_numpy(),
            "pressure": lb.total_pressure.to_numpy(), "pressure_mc": lb.pressure.to_numpy()}, lb


@pytest.mark.parametrize("fp", ["f32", "f64"])
def test_two_component_shan_chen_matches_reference(tl, fp):
    meta, arrays = load(f"mc_sc2_bgk_{fp}")
    got, lb = run(tl, meta, arrays)
    for k, v in got.items():
        ref = arrays[k]
        assert v.shape == ref.shape, (k, v.shape, ref.shape)
        assert np.isfinite(v).all(), k
        assert rel_err(v, ref) <= 1e-5, (k, rel_err(v, ref))
    # the components separate: the disc stays rich in component 0
    rho = got["rho_mc"]
    assert rho[11, 9, 0] > 0.5 > rho[0, 0, 0]


def test_two_component_mass_of_each_component_is_conserved(tl):
    meta, arrays = load("mc_sc2_bgk_f32")
    got, _ = run(tl, dict(meta, steps=200), arrays)
    m0 = np.asarray(arrays["init_rho_mc"], np.float64).sum((0, 1))
    m1 = got["rho_mc"].astype(np.float64).sum((0, 1))
    assert np.all(np.abs(m1 - m0) / m0 < 1e-5), (m0, m1)
