"""Oracle (test infrastructure only): multi-component Shan-Chen step.

A numpy restatement, in the reference's expression order, of the step its
example driver composes (cases/Bubble or two-phase separation.py:197-212)
for a lattice of nc components, each with its own populations:

    density -> pressure2 -> update_psi (ShanChenForceC2) -> psi periodic
    boundaries -> cau_SCforce (ShanChenForceC2) -> force_density -> velocity
    -> BGK collision per component -> periodic streaming

Every node is fluid (fluid_strategy true everywhere), so the adhesion term
is zero.  Nothing in the product imports this module; tests compare it with
the fixtures tests/golden/make_golden.py writes from the reference's source.
"""
import numpy as np

C = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]])  # lbm.py:44-45
W = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)


class MultiComponentSC:
    """State f[c][k] of shape (nx, ny) per component and population, in
    dtype float32 (the reference's default) or float64."""

    def __init__(self, meta, arrays):
        self.dt = np.float64 if meta.get("fp") == "f64" else np.float32
        dt = self.dt
        self.nx, self.ny = int(meta["NX"]), int(meta["NY"])
        sc = meta["sc"]
        self.nc = int(sc["components"])
        self.g = np.asarray(sc["g_coh"], np.float64).astype(dt)
        self.rho0 = [dt(p[1]) for p in sc["psi"]]
        self.w = W.astype(dt)
        self.wc = [(dt(self.w[k] * C[k, 0]), dt(self.w[k] * C[k, 1])) for k in range(9)]
        self.grav = np.asarray(meta.get("gravity", [0.0, 0.0]), np.float64).astype(dt)
        nu = np.asarray(meta["collision"]["nu"], np.float64).astype(dt)
        self.tau = [nu[c] * dt(3.0) + dt(0.5) for c in range(self.nc)]  # CollisionEngine.py:66-70
        rho = np.asarray(arrays["init_rho_mc"], dt)
        zero = np.zeros((self.nx, self.ny), dt)
        self.vel = (zero.copy(), zero.copy())
        # init_LBM: f = f2 = feq(vel, rho_c) (lbm.py:119-125)
        self.f = [self.feq(rho[:, :, c]) for c in range(self.nc)]
        self.psi = np.zeros((self.nx + 2, self.ny + 2, self.nc), dt)  # offset (-1, -1)

    # CollisionEngine.py:14-26
    def feq(self, rho):
        ux, uy = self.vel
        uv = ux * ux + uy * uy
        out = []
        for k in range(9):
            eu = self.dt(C[k, 0]) * ux + self.dt(C[k, 1]) * uy
            out.append((self.w[k] * rho) * (((1 + 3 * eu) + (4.5 * eu) * eu) - 1.5 * uv))
        return out

    def force(self, F):
        ux, uy = self.vel
        uF = ux * F[0] + uy * F[1]
        out = []
        for k in range(9):
            cF = self.dt(C[k, 0]) * F[0] + self.dt(C[k, 1]) * F[1]
            cu = self.dt(C[k, 0]) * ux + self.dt(C[k, 1]) * uy
            out.append(self.w[k] * (((3 * cF) + (9 * cF) * cu) - 3 * uF))
        return out

    def moments(self):
        dt = self.dt
        nc = self.nc
        # MacroscopicEngine.density (lbm.py:153-164)
        self.rho = []
        tot = np.zeros((self.nx, self.ny), dt)
        for c in range(nc):
            r = np.zeros((self.nx, self.ny), dt)
            for k in range(9):
                r = r + self.f[c][k]
            self.rho.append(r)
            tot = tot + r
        self.total_rho = tot
        # pressure2 (lbm.py:185-202), with the psi of the previous update
        psi_in = self.psi[1:-1, 1:-1, :]
        self.pressure_c = [np.zeros_like(tot) + (self.rho[c] + 0.5 * self.g[c, c] * (psi_in[:, :, c] * psi_in[:, :, c])) / 3.0
                           for c in range(nc)]
        p_ii = np.zeros_like(tot)
        p_ij = np.zeros_like(tot)
        for c1 in range(nc):
            p_ii = p_ii + self.pressure_c[c1]
            for c2 in range(c1 + 1, nc):
                p_ij = p_ij + (self.g[c1, c2] * psi_in[:, :, c1]) * psi_in[:, :, c2]
        self.total_pressure = p_ii + p_ij / 6.0
        # ShanChenForceC2.update_psi (ExternalForce.py:86-92), SC_psi (EOS.py:41-47)
        for c in range(nc):
            r0 = self.rho0[c]
            self.psi[1:-1, 1:-1, c] = r0 * (1.0 - np.exp(-self.rho[c] / r0))
        # PeriodicPsi_LR then PeriodicPsi_BT (SCBoundaryCondition.py:126-142)
        self.psi[0, :, :] = self.psi[self.nx, :, :]
        self.psi[self.nx + 1, :, :] = self.psi[1, :, :]
        self.psi[:, 0, :] = self.psi[:, self.ny, :]
        self.psi[:, self.ny + 1, :] = self.psi[:, 1, :]
        # ShanChenForceC2.cau_SCforce (ExternalForce.py:96-116): cohesion with
        # the other components' psi at the eight neighbours
        self.sc_force = []
        for c1 in range(nc):
            fx = np.zeros_like(tot)
            fy = np.zeros_like(tot)
            for k in range(1, 9):
                cx, cy = C[k]
                nb = self.psi[1 + cx:1 + cx + self.nx, 1 + cy:1 + cy + self.ny, :]
                for c2 in range(nc):
                    if c2 != c1:
                        fx = fx + (self.wc[k][0] * nb[:, :, c2]) * self.g[c1, c2]
                        fy = fy + (self.wc[k][1] * nb[:, :, c2]) * self.g[c1, c2]
            m = -self.psi[1:-1, 1:-1, c1]
            self.sc_force.append((m * fx, m * fy))
        # force_density (lbm.py:215-220)
        self.body_force = []
        for c in range(nc):
            frac = self.rho[c] / tot
            self.body_force.append((self.sc_force[c][0] + frac * self.grav[0],
                                    self.sc_force[c][1] + frac * self.grav[1]))
        # velocity: the mixture's (lbm.py:223-237)
        vx = np.zeros_like(tot)
        vy = np.zeros_like(tot)
        for c in range(nc):
            tx = np.zeros_like(tot)
            ty = np.zeros_like(tot)
            for k in range(9):
                tx = tx + self.f[c][k] * dt(C[k, 0])
                ty = ty + self.f[c][k] * dt(C[k, 1])
            tx = tx + 0.5 * self.body_force[c][0]
            ty = ty + 0.5 * self.body_force[c][1]
            vx = vx + tx
            vy = vy + ty
        self.vel = (vx / tot, vy / tot)

    def collide_stream(self):
        """BGKCollision.apply per component (CollisionEngine.py:101-110), then
        PeriodicAllBoundary (BoundaryCondition.py:419-432)."""
        dt = self.dt
        f2 = []
        for c in range(self.nc):
            omega = dt(1.0) / self.tau[c]
            fe = self.feq(self.rho[c])
            fo = self.force(self.body_force[c])
            cf = dt(1.0) - dt(0.5) * omega
            f2.append([(self.f[c][k] + (-omega) * (self.f[c][k] - fe[k])) + cf * fo[k] for k in range(9)])
        self.f2 = f2
        self.f = [[np.roll(f2[c][k], (int(C[k, 0]), int(C[k, 1])), axis=(0, 1)) for k in range(9)]
                  for c in range(self.nc)]

    def step(self):
        self.moments()
        self.collide_stream()

    def fields(self):
        """The comparison point: the moment prologue of the next step."""
        self.moments()
        nc = self.nc
        return {"f_mc": np.stack([np.stack(self.f[c], -1) for c in range(nc)], 2),
                "f2_mc": np.stack([np.stack(self.f2[c], -1) for c in range(nc)], 2),
                "rho_mc": np.stack(self.rho, -1), "total_rho": self.total_rho,
                "vel": np.stack(self.vel, -1), "psi_mc": self.psi.copy(),
                "sc_force_mc": np.stack([np.stack(self.sc_force[c], -1) for c in range(nc)], 2),
                "body_force_mc": np.stack([np.stack(self.body_force[c], -1) for c in range(nc)], 2),
                "pressure": self.total_pressure, "pressure_mc": np.stack(self.pressure_c, -1)}


def replay(meta, arrays, steps=None):
    run = MultiComponentSC(meta, arrays)
    for _ in range(int(meta["steps"] if steps is None else steps)):
        run.step()
    return run.fields()
