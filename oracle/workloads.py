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
