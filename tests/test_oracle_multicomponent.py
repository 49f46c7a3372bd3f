"""The multi-component Shan-Chen oracle against the reference's own source.

tests/golden/mc_sc2_bgk_{f32,f64}.npz come from make_golden.py running the
reference's taichi_lbm (LBField with two components, ShanChenForceC2,
pressure2, BGK per component with the mixture velocity, periodic psi and
stream boundaries) under the serial Taichi stand-in.  oracle/multicomponent.py
restates that step in numpy; every field at the comparison point must agree:
to rounding for f32 (the stand-in's matrix products may sum in another order)
and to 1e-12 for f64.
"""
import json

import numpy as np
import pytest

from oracle import multicomponent as MC
from tests.cases import ROOT

FIELDS = ("f_mc", "f2_mc", "rho_mc", "total_rho", "vel", "psi_mc", "sc_force_mc", "body_force_mc",
          "pressure", "pressure_mc")


def load(name):
    d = np.load(f"{ROOT}/tests/golden/{name}.npz")
    return json.loads(str(d["meta"])), {k: d[k] for k in d.files if k != "meta"}


@pytest.mark.parametrize("fp,tol", [("f32", 2e-6), ("f64", 1e-12)])
def test_two_component_shan_chen_matches_reference(fp, tol):
    meta, arrays = load(f"mc_sc2_bgk_{fp}")
    got = MC.replay(meta, arrays)
    for k in FIELDS:
        a, b = np.asarray(got[k], np.float64), np.asarray(arrays[k], np.float64)
        assert a.shape == b.shape, (k, a.shape, b.shape)
        err = np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)
        assert err <= tol, (k, err)


def test_two_component_mass_of_each_component_is_conserved():
    """Periodic, no sources: each component's mass is constant (FP64 run)."""
    meta, arrays = load("mc_sc2_bgk_f64")
    run = MC.MultiComponentSC(meta, arrays)
    m0 = [float(np.sum(run.f[c])) for c in range(run.nc)]
    for _ in range(20):
        run.step()
    m1 = [float(np.sum(run.f[c])) for c in range(run.nc)]
    assert np.allclose(m0, m1, rtol=1e-13, atol=0.0)
