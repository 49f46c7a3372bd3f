"""Known-answer checks of the oracle (FP64): equilibrium moments, rest-state
fixed point, mass conservation, TRT/MRT reductions to BGK, exact TRT
Poiseuille flow, and the Shan-Chen coexistence densities tabulated in the
reference's two-phase example (cases/Bubble or two-phase separation.py:48-68)."""
import numpy as np
import pytest

from oracle import oracle as O


def periodic_case(nx, ny, model="bgk", nu=1.0 / 6.0, magic=0.25, nu_bulk=None, steps=10,
                  rho=None, vel=None, gravity=(0.0, 0.0), walls_y=False, sc=None, fp="f64", diag=None):
    nodes = np.argwhere(np.ones((nx, ny), bool)).astype(np.int32)
    bcs = [{"name": "fluid", "kind": "fluid"}, {"name": "stream", "kind": "periodic"}]
    arrays = {"mask": np.ones((nx, ny), np.int32), "g_fluid": nodes, "g_stream": nodes}
    if walls_y:
        wall = nodes[(nodes[:, 1] == 0) | (nodes[:, 1] == ny - 1)]
        bcs.append({"name": "wall", "kind": "bounceback"})
        arrays["g_wall"] = wall
    arrays["init_rho"] = np.ones((nx, ny)) if rho is None else rho
    arrays["init_vel"] = np.zeros((nx, ny, 2)) if vel is None else vel
    coll = {"model": model, "nu": [nu], "tau_min": 0.5000001, "tau_max": 4.0, "magic": [magic],
            "nu_bulk": [nu if nu_bulk is None else nu_bulk], "mrt_diag": diag}
    meta = {"name": "t", "NX": nx, "NY": ny, "fp": fp, "bcs": bcs, "collision": coll,
            "fluid_model": ["newtonian", nu], "gravity": list(gravity), "steps": steps,
            "step_kind": "shanchen" if sc else "standard", "sc": sc,
            "psi_bcs": ["periodic_lr", "periodic_bt"] if sc else []}
    if sc:
        arrays["T"] = np.ones((nx, ny))
    return meta, arrays


def test_equilibrium_moments(built):
    rng = np.random.default_rng(1)
    rho = 1 + 0.1 * rng.random((6, 5))
    vel = 0.05 * (rng.random((6, 5, 2)) - 0.5)
    meta, arrays = periodic_case(6, 5, rho=rho, vel=vel, steps=0)
    o = O.Oracle(6, 5, True)
    o.field("rho")[...] = rho
    o.field("vel")[...] = vel
    o.call("init_lbm", arrays["g_fluid"])
    f = o.field("f")
    c = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]])
    assert np.allclose(f.sum(-1), rho, rtol=0, atol=1e-14)
    assert np.allclose(f @ c, rho[..., None] * vel, rtol=0, atol=1e-14)


def test_rest_state_is_fixed_point(built):
    for model in ("bgk", "trt", "mrt"):
        meta, arrays = periodic_case(8, 6, model=model, steps=50)
        out = O.replay(meta, arrays)
        assert np.abs(out["rho"] - 1).max() < 1e-14
        assert np.abs(out["vel"]).max() < 1e-13


def test_periodic_mass_conservation(built):
    rng = np.random.default_rng(2)
    rho = 1 + 0.05 * rng.random((16, 12))
    vel = 0.04 * (rng.random((16, 12, 2)) - 0.5)
    for model in ("bgk", "trt", "mrt"):
        meta, arrays = periodic_case(16, 12, model=model, rho=rho, vel=vel, steps=200)
        out = O.replay(meta, arrays)
        m0 = rho.sum()
        assert abs(out["f"].sum() - m0) / m0 < 1e-13


def test_trt_with_equal_rates_is_bgk(built):
    rng = np.random.default_rng(3)
    rho = 1 + 0.05 * rng.random((12, 10))
    vel = 0.04 * (rng.random((12, 10, 2)) - 0.5)
    nu = 0.1
    tau = 3 * nu + 0.5
    magic = (tau - 0.5) ** 2  # tau_minus = magic / (tau - 1/2) + 1/2 = tau
    a = O.replay(*periodic_case(12, 10, "bgk", nu=nu, rho=rho, vel=vel, steps=40, gravity=(1e-5, 0)))
    b = O.replay(*periodic_case(12, 10, "trt", nu=nu, magic=magic, rho=rho, vel=vel, steps=40,
                                gravity=(1e-5, 0)))
    assert np.abs(a["f"] - b["f"]).max() < 1e-13


def test_mrt_with_equal_rates_is_bgk(built):
    rng = np.random.default_rng(4)
    rho = 1 + 0.05 * rng.random((12, 10))
    vel = 0.04 * (rng.random((12, 10, 2)) - 0.5)
    nu = 0.1
    s = 1.0 / (3 * nu + 0.5)
    a = O.replay(*periodic_case(12, 10, "bgk", nu=nu, rho=rho, vel=vel, steps=40))
    b = O.replay(*periodic_case(12, 10, "mrt", nu=nu, rho=rho, vel=vel, steps=40, diag=[s] * 9))
    assert np.abs(a["f"] - b["f"]).max() < 1e-13


def test_trt_poiseuille_is_exact(built):
    """Body-force-driven channel with half-way bounce-back walls at y = -1/2
    and y = H - 1/2: TRT with magic 3/16 gives the parabola to round-off."""
    # The reference's neighbor table is not periodic, so a BounceBackWall
    # node at an x edge would also bounce its x links; the table is patched
    # to wrap in x here so the walls bounce only the y links.
    nx, ny, g, nu = 2, 17, 1e-6, 0.1
    o = O.Oracle(nx, ny, True)
    o.L.orc_neighbor_classify(o.h)
    nb = o.field("neighbor")
    c = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]])
    for i in range(nx):
        for j in range(ny):
            for k in range(9):
                j2 = j - c[k, 1]
                nb[i, j, k] = ((i - c[k, 0]) % nx, j2) if 0 <= j2 < ny else (-1, -1)
    nodes = np.argwhere(np.ones((nx, ny), bool)).astype(np.int32)
    wall = nodes[(nodes[:, 1] == 0) | (nodes[:, 1] == ny - 1)]
    o.field("gravity")[...] = (g, 0.0)
    o.field("rho")[...] = 1.0
    o.call("trt_init_tau", nodes, nu, 3.0 / 16.0)
    o.call("init_lbm", nodes)

    def moments():
        o.call("density", nodes)
        o.call("pressure", nodes, 0, 0.0)
        o.call("force_density", nodes)
        o.call("velocity", nodes)

    for _ in range(6000):
        moments()
        o.call("trt_apply", nodes)
        o.call("bc_periodic", nodes)
        o.call("bc_bounceback", wall)
    moments()
    y = np.arange(ny) + 0.5
    exact = g / (2 * nu) * y * (ny - y)
    u = o.field("vel")[0, :, 0].copy()
    assert np.abs(u - exact).max() / exact.max() < 1e-6


@pytest.mark.parametrize("idx", [15, 17])
def test_shan_chen_coexistence_table(built, idx):
    """Flat liquid slab in gas with psi = 1 - exp(-rho): the equilibrium
    densities approach the reference example's coexistence table."""
    G = [-8, -7.8, -7.6, -7.4, -7.2, -7, -6.8, -6.6, -6.4, -6.2, -6, -5.8, -5.6, -5.4, -5.2, -5, -4.8, -4.6][idx]
    table = {15: (0.156413030238316, 1.93244248895799), 17: (0.228058754735636, 1.59001518629020)}[idx]
    ny = 64
    rho = np.full((2, ny), table[0])
    rho[:, ny // 4: 3 * ny // 4] = table[1]
    meta, arrays = periodic_case(2, ny, "bgk", nu=0.5 / 3.0, rho=rho, steps=20000,
                                 sc={"g_coh": float(G), "psi": ["sc", 1.0]})
    out = O.replay(meta, arrays)
    r = out["rho"][0]
    gas, liq = r.min(), r.max()
    # The table is the mechanical-stability solution; with Guo forcing (what
    # the reference uses, CollisionEngine.py:21-25) the pseudopotential model
    # is known to land below it on the gas branch (measured: -24 % at G=-5,
    # -11 % at G=-4.6) and within 2.5 % on the liquid branch.
    assert -0.26 < (gas - table[0]) / table[0] < 0.0
    assert abs(liq - table[1]) / table[1] < 0.03
