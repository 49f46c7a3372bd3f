"""Case descriptions of the benchmark workloads for the oracle (numpy only,
no GPU): the cylinder channel used by bench.py, built with the same
definitions as the drop-in workload builder taichi_lbm.workloads."""
import numpy as np

C = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]])


def cylinder_channel_case(nx, ny, radius, cx, cy, tau, umax, model="bgk", magic=0.25, mrt_s=None,
                          steps=1):
    """Channel, walls on every edge (bounce-back on missing links), periodic
    stream carrier, parabolic VelocityEquilibrium inlet (i = 0, direction 3),
    PressureNEEM outlet (i = NX-1, rho = 1, direction 1)."""
    x, y, r = np.float32(cx), np.float32(cy), np.float32(radius)
    dx = np.arange(nx, dtype=np.float32)[:, None] - x
    dy = np.arange(ny, dtype=np.float32)[None, :] - y
    mask = np.where(dx * dx + dy * dy < r * r, -1, 1).astype(np.int32)
    fluid = mask == 1
    missing = np.zeros((nx, ny), bool)
    pad = np.pad(fluid, 1, constant_values=False)
    for k in range(9):
        # source of link k is (i - cx_k, j - cy_k)
        src = pad[1 - C[k, 0]:1 - C[k, 0] + nx, 1 - C[k, 1]:1 - C[k, 1] + ny]
        missing |= ~src
    wall = fluid & missing
    inlet = fluid.copy()
    inlet[1:] = False
    outlet = fluid.copy()
    outlet[:-1] = False
    nodes = lambda m: np.argwhere(m).astype(np.int32)  # noqa: E731
    g_in = nodes(inlet)
    yv = g_in[:, 1] + 0.5
    u_in = np.stack([4.0 * umax * yv * (ny - yv) / (ny * ny), np.zeros_like(yv)], 1).astype(np.float32)
    nu = (tau - 0.5) / 3.0
    bcs = [{"name": "fluid", "kind": "fluid"}, {"name": "periodic", "kind": "periodic"},
           {"name": "wall", "kind": "bounceback"},
           {"name": "inlet", "kind": "velocity_eq", "direction": 3, "velocity": [umax, 0.0]},
           {"name": "outlet", "kind": "pressure_neem", "direction": 1, "rho": 1.0}]
    g_f = nodes(fluid)
    arrays = {"mask": mask, "g_fluid": g_f, "g_periodic": g_f, "g_wall": nodes(wall),
              "g_inlet": g_in, "u_inlet": u_in, "g_outlet": nodes(outlet),
              "init_rho": fluid.astype(np.float32), "init_vel": np.zeros((nx, ny, 2), np.float32)}
    coll = {"model": model, "nu": [nu], "tau_min": 0.5000001, "tau_max": 4.0, "magic": [magic],
            "nu_bulk": [nu], "mrt_diag": None if mrt_s is None else list(mrt_s)}
    meta = {"name": f"cylinder_{nx}x{ny}", "NX": nx, "NY": ny, "fp": "f32", "bcs": bcs,
            "collision": coll, "fluid_model": ["newtonian", nu], "gravity": [0.0, 0.0],
            "steps": steps, "step_kind": "standard", "sc": None, "psi_bcs": []}
    return meta, arrays


def contraction_case(nx=2048, ny=512, outlet_h=128, n=1.0, re=20.0, umax=0.02, magic=0.25,
                     tau_clamp=(0.505, 2.0), steps=1, fp="f32"):
    """The power-law planar contraction of taichi_lbm.workloads.contraction_channel
    (solid above and below an outlet section `outlet_h` high for x >= NX/2, the
    reference's open-rectangle mask rule BoundaryCondition.py:464-469 in f32),
    TRT, parabolic inlet over the full height, PressureNEEM outlet."""
    lo, hi = (ny - outlet_h) // 2, (ny + outlet_h) // 2
    i = np.arange(nx)[:, None]
    j = np.arange(ny)[None, :]
    f32 = np.float32
    solid = np.zeros((nx, ny), bool)
    for x0, x1, y0, y1 in ((nx // 2 - 1, nx + 1, -1, lo), (nx // 2 - 1, nx + 1, hi - 1, ny + 1)):
        solid |= (i < f32(x1)) & (i > f32(x0)) & (j < f32(y1)) & (j > f32(y0))
    mask = np.where(solid, -1, 1).astype(np.int32)
    m = umax ** (2.0 - n) * float(outlet_h) ** n / re
    nu0 = m * (umax / outlet_h) ** (n - 1.0)
    tau = min(max(0.5 + 3.0 * nu0, tau_clamp[0]), tau_clamp[1])
    meta, arrays = _channel_case(mask, nx, ny, tau, umax, "trt", magic, None, steps)
    meta["collision"]["tau_min"], meta["collision"]["tau_max"] = float(tau_clamp[0]), float(tau_clamp[1])
    meta["fluid_model"] = ["powerlaw", float(m), float(n)]
    meta["step_kind"] = "powerlaw"
    meta["fp"] = fp
    return meta, arrays


def _channel_case(mask, nx, ny, tau, umax, model, magic, mrt_s, steps):
    fluid = mask == 1
    missing = np.zeros((nx, ny), bool)
    pad = np.pad(fluid, 1, constant_values=False)
    for k in range(9):
        src = pad[1 - C[k, 0]:1 - C[k, 0] + nx, 1 - C[k, 1]:1 - C[k, 1] + ny]
        missing |= ~src
    wall = fluid & missing
    inlet = fluid.copy()
    inlet[1:] = False
    outlet = fluid.copy()
    outlet[:-1] = False
    nodes = lambda m: np.argwhere(m).astype(np.int32)  # noqa: E731
    g_in = nodes(inlet)
    yv = np.clip(g_in[:, 1] + 0.5, 0.0, float(ny))
    h = float(ny)
    u_in = np.stack([4.0 * umax * yv * (h - yv) / (h * h), np.zeros_like(yv)], 1).astype(np.float32)
    nu = (tau - 0.5) / 3.0
    bcs = [{"name": "fluid", "kind": "fluid"}, {"name": "periodic", "kind": "periodic"},
           {"name": "wall", "kind": "bounceback"},
           {"name": "inlet", "kind": "velocity_eq", "direction": 3, "velocity": [umax, 0.0]},
           {"name": "outlet", "kind": "pressure_neem", "direction": 1, "rho": 1.0}]
    g_f = nodes(fluid)
    arrays = {"mask": mask, "g_fluid": g_f, "g_periodic": g_f, "g_wall": nodes(wall),
              "g_inlet": g_in, "u_inlet": u_in, "g_outlet": nodes(outlet),
              "init_rho": fluid.astype(np.float32), "init_vel": np.zeros((nx, ny, 2), np.float32)}
    coll = {"model": model, "nu": [nu], "tau_min": 0.5000001, "tau_max": 4.0, "magic": [magic],
            "nu_bulk": [nu], "mrt_diag": None if mrt_s is None else list(mrt_s)}
    meta = {"name": f"channel_{nx}x{ny}", "NX": nx, "NY": ny, "fp": "f32", "bcs": bcs,
            "collision": coll, "fluid_model": ["newtonian", nu], "gravity": [0.0, 0.0],
            "steps": steps, "step_kind": "standard", "sc": None, "psi_bcs": []}
    return meta, arrays
