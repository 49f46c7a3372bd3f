"""The immersed-boundary oracle against the reference's own ibm.py.

tests/golden/ibm_circle_bgk_f32.npz comes from make_golden.py running the
reference's SphereIB, IBDEMCouplerEngine and IBEngine (two multi-direct
forcing iterations between the velocity and the BGK collision, a periodic
box driven by gravity past one circle of IB nodes) under the serial Taichi
stand-in; oracle/ibm.py restates that step.  Every field, the IB nodes'
velocities and forces and the particle resultant must agree.
"""
import json

import numpy as np

from oracle import ibm as IB
from tests.cases import ROOT

FIELDS = ("f", "f2", "rho", "vel", "body_force", "ib_pos", "ib_vel", "ib_force", "ib_force_temp",
          "sphere_force", "sphere_torque")


def test_immersed_circle_matches_reference():
    d = np.load(f"{ROOT}/tests/golden/ibm_circle_bgk_f32.npz")
    meta = json.loads(str(d["meta"]))
    arrays = {k: d[k] for k in d.files if k != "meta"}
    got = IB.replay(meta, arrays)
    assert int(arrays["ib_count"]) == got["ib_pos"].shape[0]
    for k in FIELDS:
        a, b = np.asarray(got[k], np.float64), np.asarray(arrays[k], np.float64)
        assert a.shape == b.shape, (k, a.shape, b.shape)
        err = np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)
        assert err <= 1e-6, (k, err)


def test_forcing_drives_the_nodes_toward_rest():
    """More multi-direct forcing iterations leave a smaller slip velocity at
    the IB nodes (the circle is at rest)."""
    d = np.load(f"{ROOT}/tests/golden/ibm_circle_bgk_f32.npz")
    meta = json.loads(str(d["meta"]))
    arrays = {k: d[k] for k in d.files if k != "meta"}
    slips = []
    for mdf in (1, 4):
        m = dict(meta, ibm=dict(meta["ibm"], mdf=mdf))
        run = IB.IBBox(m, arrays)
        for _ in range(20):
            run.step()
        run.moments()
        c = run.circle
        v = [np.hypot(*sum(np.array([run.vx[i, j], run.vy[i, j]]) * w for i, j, w in c.stencil(k)))
             for k in range(c.n)]
        slips.append(max(v))
    assert slips[1] < slips[0]
