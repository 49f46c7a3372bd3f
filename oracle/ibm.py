"""Oracle (test infrastructure only): immersed-boundary step.

A numpy restatement of the reference's immersed-boundary coupling
(taichi_lbm/ibm.py) inside a single-component BGK step on a periodic box:

    density -> pressure -> force_density -> velocity
    -> IBEngine.MultiDirectForcingLoop (reset node forces; `mdf` times:
       InterpolateBodyVelocities, SpreadBodyForces)
    -> IBEngine.ComputeParticleForce -> BGK collision -> periodic streaming

for one circle of IB nodes placed by SphereIB / IBDEMCouplerEngine.  The node
loops run in node order, the serial order the fixtures were written in (the
reference's parallel loops add to shared grid nodes and, in
ComputeParticleForce, reset the particle's sum once per node, so the
resultant it reports is the last node's force: ibm.py:171-185).  Nothing in
the product imports this module.
"""
import math

import numpy as np

C = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]])  # lbm.py:44-45
W = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
F32 = np.float32


class IBCircle:
    """One static circle: node positions as SphereIB.computer_IB_nodes_pos
    (ibm.py:69-78) evaluates them, rounded to the f32 node field."""

    def __init__(self, center, radius, nx, ny, angle=0.0):
        self.center = np.array(center, F32)
        self.radius = F32(radius)
        # SphereIB.init_IB_nodes (ibm.py:57-67): NUMIB_cof = 1
        self.n = int(np.round(F32(math.pi * 2) * self.radius))
        pos = np.zeros((self.n, 2), F32)
        a = F32(angle)
        for k in range(self.n):
            ang = 2.0 * math.pi * k / self.n
            xref = float(self.radius) * float(np.cos(ang))
            yref = float(self.radius) * float(np.sin(ang))
            pos[k, 0] = float(self.center[0]) + xref * float(np.cos(a)) - yref * float(np.sin(a))
            pos[k, 1] = float(self.center[1]) + xref * float(np.sin(a)) + yref * float(np.cos(a))
        self.pos = pos
        self.vel_desired = np.zeros((self.n, 2), F32)
        self.vel = np.zeros((self.n, 2), F32)
        self.force = np.zeros((self.n, 2), F32)
        self.force_temp = np.zeros((self.n, 2), F32)
        # IBDEMCouplerEngine.CheckPos (ibm.py:92-109): the circle lies inside
        d = 2 * float(self.radius)
        assert (center[0] - d >= 0 and center[0] + d <= nx - 1 and center[1] - d >= 0
                and center[1] + d <= ny - 1), "the restated case keeps the circle inside"

    def stencil(self, k):
        """Grid nodes around node k and their weights (ibm.py:187-199)."""
        p = self.pos[k]
        xb, yb = int(np.floor(p[0])), int(np.floor(p[1]))
        xt, yt = int(np.ceil(p[0])), int(np.ceil(p[1]))
        for ix in range(xb, xt + 1):
            for iy in range(yb, yt + 1):
                w = (F32(1.0) - np.abs(p[0] - F32(ix))) * (F32(1.0) - np.abs(p[1] - F32(iy)))
                yield ix, iy, w


class IBBox:
    def __init__(self, meta, arrays):
        self.nx, self.ny = int(meta["NX"]), int(meta["NY"])
        ib = meta["ibm"]
        self.mdf = int(ib["mdf"])
        self.circle = IBCircle(ib["center"], ib["radius"], self.nx, self.ny)
        self.g = np.asarray(meta["gravity"], np.float64).astype(F32)
        nu = F32(meta["collision"]["nu"][0])
        self.tau = nu * F32(3.0) + F32(0.5)
        self.w = W.astype(F32)
        rho = np.asarray(arrays["init_rho"], F32)
        z = np.zeros((self.nx, self.ny), F32)
        self.vx, self.vy = z.copy(), z.copy()
        self.f = self.feq(rho)
        self.sphere_force = np.zeros(2, F32)
        self.sphere_torque = F32(0.0)

    def feq(self, rho):  # CollisionEngine.py:14-18
        uv = self.vx * self.vx + self.vy * self.vy
        out = []
        for k in range(9):
            eu = F32(C[k, 0]) * self.vx + F32(C[k, 1]) * self.vy
            out.append((self.w[k] * rho) * (((1 + 3 * eu) + (4.5 * eu) * eu) - 1.5 * uv))
        return out

    def moments(self):
        z = np.zeros((self.nx, self.ny), F32)
        rho = z.copy()
        for k in range(9):  # lbm.py:153-164
            rho = rho + self.f[k]
        self.rho = rho
        self.total_rho = z + rho
        # force_density (lbm.py:215-220); no Shan-Chen force
        frac = self.rho / self.total_rho
        self.fx = z + frac * self.g[0]
        self.fy = z + frac * self.g[1]
        tx, ty = z.copy(), z.copy()  # velocity (lbm.py:223-237)
        for k in range(9):
            tx = tx + self.f[k] * F32(C[k, 0])
            ty = ty + self.f[k] * F32(C[k, 1])
        tx = tx + 0.5 * self.fx
        ty = ty + 0.5 * self.fy
        self.vx = (z + tx) / self.total_rho
        self.vy = (z + ty) / self.total_rho

    def forcing(self):
        """IBEngine.MultiDirectForcingLoop and ComputeParticleForce (ibm.py:171-253)."""
        c = self.circle
        c.force[:] = 0
        for _ in range(self.mdf):
            for k in range(c.n):  # InterpolateBodyVelocities
                v = np.zeros(2, F32)
                for ix, iy, w in c.stencil(k):
                    v = v + np.array([self.vx[ix, iy], self.vy[ix, iy]], F32) * w
                c.vel[k] = v
                fc = 2 * (c.vel_desired[k] - v)
                c.force_temp[k] = fc
                c.force[k] = c.force[k] + fc
            for k in range(c.n):  # SpreadBodyForces
                for ix, iy, w in c.stencil(k):
                    ft = np.zeros(2, F32) + c.force_temp[k] * w
                    r2 = self.total_rho[ix, iy] * F32(2.0)
                    self.vx[ix, iy] = self.vx[ix, iy] + ft[0] / r2
                    self.vy[ix, iy] = self.vy[ix, iy] + ft[1] / r2
                    self.fx[ix, iy] = self.fx[ix, iy] + (ft[0] * self.rho[ix, iy]) / self.total_rho[ix, iy]
                    self.fy[ix, iy] = self.fy[ix, iy] + (ft[1] * self.rho[ix, iy]) / self.total_rho[ix, iy]
        for k in range(c.n):  # ComputeParticleForce: the sum restarts at every node
            fx, fy = c.force[k]
            rx, ry = c.pos[k] - c.center
            self.sphere_torque = F32(0.0) + (fx * ry - fy * rx)
            self.sphere_force = np.array([F32(0.0) + fx, F32(0.0) + fy], F32)

    def collide_stream(self):
        """BGK with Guo forcing (CollisionEngine.py:101-110), periodic stream."""
        omega = F32(1.0) / self.tau
        fe = self.feq(self.rho)
        uF = self.vx * self.fx + self.vy * self.fy
        f2 = []
        for k in range(9):
            cF = F32(C[k, 0]) * self.fx + F32(C[k, 1]) * self.fy
            cu = F32(C[k, 0]) * self.vx + F32(C[k, 1]) * self.vy
            fo = self.w[k] * (((3 * cF) + (9 * cF) * cu) - 3 * uF)
            f2.append((self.f[k] + (-omega) * (self.f[k] - fe[k])) + (F32(1.0) - F32(0.5) * omega) * fo)
        self.f2 = f2
        self.f = [np.roll(f2[k], (int(C[k, 0]), int(C[k, 1])), axis=(0, 1)) for k in range(9)]

    def step(self):
        self.moments()
        self.forcing()
        self.collide_stream()


def replay(meta, arrays, steps=None):
    run = IBBox(meta, arrays)
    for _ in range(int(meta["steps"] if steps is None else steps)):
        run.step()
    c = run.circle
    out = {"ib_pos": c.pos.copy(), "ib_vel": c.vel.copy(), "ib_force": c.force.copy(),
           "ib_force_temp": c.force_temp.copy(), "sphere_force": run.sphere_force.copy(),
           "sphere_torque": np.array(run.sphere_torque)}
    run.moments()  # the comparison point: the next step's moment prologue
    out.update({"f": np.stack(run.f, -1), "f2": np.stack(run.f2, -1), "rho": run.rho,
                "vel": np.stack([run.vx, run.vy], -1), "body_force": np.stack([run.fx, run.fy], -1)})
    return out
