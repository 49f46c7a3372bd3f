"""Immersed-boundary coupling (taichi_lbm/ibm.py).

Circles of IB nodes (SphereIB) placed by a DEM coupler (IBDEMCouplerEngine)
and multi-direct forcing between the velocity and the collision (IBEngine):
the same classes, constructors, methods and argument names as the reference.
The node loops that touch the lattice run on the GPU (lbm_ibm_interpolate,
lbm_ibm_spread); node placement and the per-particle sums are host work on
a few hundred nodes.

Semantics kept from the reference:
* a particle's nodes are the insiders of its circle: all of them when the
  circle (with a margin of one diameter) lies inside the lattice, else those
  strictly inside (ibm.py:92-141);
* ComputeParticleForce resets the particle's force and torque once per
  insider node before adding that node's share (ibm.py:171-185), so the
  resultant it reports is that of the last node; the loop runs in insider
  order, the serial schedule of the reference's loop.
"""
import ctypes
import math

import numpy as np
import torch

from . import _capi
from .fields import Scalar0D
from .lbm import stream_handle

F32 = np.float32


class IBMNodes:
    """Field names of an IB node (ibm.py:7-14); SphereIB.IBNodes holds them."""
    fields = ("pos", "vel", "vel_desired", "force", "force_temp", "mask_insiderDomain")


class Sphere:
    """Field names of a particle (ibm.py:16-25); SphereIB.Sphere holds them."""
    fields = ("id", "pos", "vel", "force", "torque", "radius", "angle", "NumIB")


class _HostArray:
    """A host struct member with the field API the reference's callers use."""

    def __init__(self, a):
        self.arr = a

    def to_numpy(self):
        return self.arr.copy()

    def from_numpy(self, a):
        self.arr[...] = a

    def __getitem__(self, k):
        return self.arr[k]

    def __setitem__(self, k, v):
        self.arr[k] = v


class _Spheres:
    """Particles as struct-of-arrays on the host: Sphere.force.to_numpy(), etc."""

    def __init__(self, n):
        self.id = _HostArray(np.zeros(n, np.int32))
        self.pos = _HostArray(np.zeros((n, 2), F32))
        self.vel = _HostArray(np.zeros((n, 2), F32))
        self.force = _HostArray(np.zeros((n, 2), F32))
        self.torque = _HostArray(np.zeros(n, F32))
        self.radius = _HostArray(np.zeros(n, F32))
        self.angle = _HostArray(np.zeros(n, F32))
        self.NumIB = _HostArray(np.zeros(n, np.int32))


class _DeviceArray:
    def __init__(self, t):
        self.t = t

    def to_numpy(self):
        return self.t.cpu().numpy()

    def from_numpy(self, a):
        self.t.copy_(torch.as_tensor(np.asarray(a, F32)))


class _Nodes:
    """IB nodes as [Max_Number][Max_NumIB][2] float32 device tensors."""

    def __init__(self, m, n, device):
        shape = (m, n, 2)
        for name in ("pos", "vel", "vel_desired", "force", "force_temp"):
            setattr(self, name, _DeviceArray(torch.zeros(shape, dtype=torch.float32, device=device)))
        self.mask_insiderDomain = _DeviceArray(torch.zeros((m, n), dtype=torch.int32, device=device))


class SphereIB:
    def __init__(self, Max_Number, Max_NumIB, device="cuda"):
        self.Max_Number = int(Max_Number)
        self.Max_NumIB = int(Max_NumIB)
        self.num = Scalar0D(0)
        self.NUMIB_cof = 1
        self.device = torch.device(device)
        self.Sphere = _Spheres(self.Max_Number)
        self.IBNodes = _Nodes(self.Max_Number, self.Max_NumIB, self.device)
        self.IBNodeInsiderGroup = _HostArray(np.zeros((self.Max_Number * self.Max_NumIB, 2), np.int32))
        self.IBInsiderCount = Scalar0D(0)

    def init_Balls(self, num, id_np, pos_np, vel_np, force_np, torque_np, radius_np, angle_np):
        """ibm.py:43-54"""
        self.num[None] = int(num)
        s = self.Sphere
        for m in range(self.num[None]):
            s.id[m] = id_np[m]
            s.pos[m] = pos_np[m]
            s.vel[m] = vel_np[m]
            s.force[m] = force_np[m]
            s.torque[m] = torque_np[m]
            s.radius[m] = radius_np[m]
            s.angle[m] = angle_np[m]

    def init_IB_nodes(self):
        """ibm.py:57-67: NumIB = round(2 pi r / NUMIB_cof) nodes on the circle."""
        s = self.Sphere
        pos = self.IBNodes.pos.t.cpu().numpy()
        for m in range(self.num[None]):
            numib = int(np.round(F32(math.pi * 2) * s.radius[m] / self.NUMIB_cof))
            if numib > self.Max_NumIB:
                raise ValueError(f"particle {m} needs {numib} IB nodes, Max_NumIB is {self.Max_NumIB}")
            s.NumIB[m] = numib
            for n in range(numib):
                angle = 2.0 * math.pi * n / numib
                pos[m, n, 0] = float(s.pos[m][0]) + float(s.radius[m]) * float(np.cos(angle))
                pos[m, n, 1] = float(s.pos[m][1]) + float(s.radius[m]) * float(np.sin(angle))
        self.IBNodes.pos.from_numpy(pos)

    def computer_IB_nodes_pos(self, m, n):
        """ibm.py:69-78: node n of particle m, turned by the particle's angle
        (evaluated in double, stored as float32 like the reference's field)."""
        s = self.Sphere
        angle = 2.0 * math.pi * n / int(s.NumIB[m])
        xref = float(s.radius[m]) * float(np.cos(angle))
        yref = float(s.radius[m]) * float(np.sin(angle))
        a = s.angle[m]
        ca, sa = float(np.cos(a)), float(np.sin(a))
        return np.array([float(s.pos[m][0]) + xref * ca - yref * sa,
                         float(s.pos[m][1]) + xref * sa + yref * ca], F32)

    def reset_force(self):
        """ibm.py:80-84"""
        self.IBNodes.force.t.zero_()

    # the insider nodes as flat indices m * Max_NumIB + n, in insider order
    def _insiders(self):
        g = self.IBNodeInsiderGroup.arr[:self.IBInsiderCount[None]]
        idx = g[:, 0].astype(np.int64) * self.Max_NumIB + g[:, 1]
        return torch.as_tensor(idx, device=self.device)


class IBDEMCouplerEngine:
    def __init__(self, lb_field):
        self.NX = lb_field.NX
        self.NY = lb_field.NY

    def CheckPos(self, pos, diameter):
        """ibm.py:92-109: 1 inside (with a margin of one diameter), 0 outside, 2 crossing."""
        x_min, x_max = pos[0] - diameter, pos[0] + diameter
        y_min, y_max = pos[1] - diameter, pos[1] + diameter
        nx, ny = self.NX - 1, self.NY - 1
        if x_min >= 0 and x_max <= nx and y_min >= 0 and y_max <= ny:
            return 1
        if x_max < 0 or x_min > nx or y_max < 0 or y_min > ny:
            return 0
        return 2

    def InDomain(self, pos):
        """ibm.py:111-117"""
        return 1 if (0 < pos[0] < self.NX - 1 and 0 < pos[1] < self.NY - 1) else 0

    def SphereIBUpdate(self, sphere_field):
        """ibm.py:120-141: node positions, desired velocities and the insider list."""
        s = sphere_field.Sphere
        pos = sphere_field.IBNodes.pos.t.cpu().numpy()
        vd = sphere_field.IBNodes.vel_desired.t.cpu().numpy()
        group = sphere_field.IBNodeInsiderGroup.arr
        group[:] = 0
        count = 0
        for m in range(sphere_field.num[None]):
            flag = self.CheckPos(s.pos[m], 2 * s.radius[m])
            if flag == 0:
                continue
            for n in range(int(s.NumIB[m])):
                pos[m, n] = sphere_field.computer_IB_nodes_pos(m, n)
                vd[m, n] = s.vel[m]
                if flag == 1 or self.InDomain(pos[m, n]):
                    group[count] = (m, n)
                    count += 1
        sphere_field.IBInsiderCount[None] = count
        sphere_field.IBNodes.pos.from_numpy(pos)
        sphere_field.IBNodes.vel_desired.from_numpy(vd)

    def SphereInfoUpdata(self, sphere_field, pos_np, vel_np, angle_np):
        """ibm.py:143-150"""
        for m in range(sphere_field.num[None]):
            sphere_field.Sphere.pos[m] = pos_np[m]
            sphere_field.Sphere.vel[m] = vel_np[m]
            sphere_field.Sphere.angle[m] = angle_np[m]
        self.SphereIBUpdate(sphere_field)

    def GetSphereForce(self, sphere_field):
        return np.array(sphere_field.Sphere.force.to_numpy(), dtype=np.float64)[:sphere_field.num[None], :]

    def GetSphereTorque(self, sphere_field):
        return np.array(sphere_field.Sphere.torque.to_numpy(), dtype=np.float64)[:sphere_field.num[None]]


class IBEngine:
    def __init__(self, MDFIteration):
        self.MDFIteration = int(MDFIteration)

    def _nodes(self, sphere_field):
        """Compact device copies of the insider nodes and their struct."""
        idx = sphere_field._insiders()
        N = sphere_field.IBNodes
        flat = {k: getattr(N, k).t.view(-1, 2) for k in ("pos", "vel", "vel_desired", "force", "force_temp")}
        c = {k: v.index_select(0, idx).contiguous() for k, v in flat.items()}
        s = _capi.LbmIBNodes()
        s.n = int(idx.numel())
        for k, v in c.items():
            setattr(s, k, v.data_ptr())
        return idx, flat, c, s

    def ComputeParticleForce(self, sphere_field):
        """ibm.py:171-185, in insider order: the particle's sum restarts at every node."""
        g = sphere_field.IBNodeInsiderGroup.arr[:sphere_field.IBInsiderCount[None]]
        force = sphere_field.IBNodes.force.to_numpy()
        pos = sphere_field.IBNodes.pos.to_numpy()
        s = sphere_field.Sphere
        for m, n in g:
            fx, fy = force[m, n]
            rx, ry = pos[m, n] - s.pos[m]
            s.torque[m] = F32(0.0) + (fx * ry - fy * rx)
            s.force[m] = (F32(0.0) + fx, F32(0.0) + fy)

    def InterpolateBodyVelocities(self, sphere_field, lb_filed):
        """ibm.py:201-223 (lbm_ibm_interpolate)"""
        lb_filed._sync_fused()
        idx, flat, c, s = self._nodes(sphere_field)
        if s.n == 0:
            return
        L = lb_filed._lattice()
        _capi.call("lbm_ibm_interpolate", ctypes.byref(L), ctypes.byref(s), stream_handle())
        for k in ("vel", "force", "force_temp"):
            flat[k].index_copy_(0, idx, c[k])

    def SpreadBodyForces(self, sphere_field, lb_filed):
        """ibm.py:225-246 (lbm_ibm_spread)"""
        lb_filed._sync_fused()
        idx, flat, c, s = self._nodes(sphere_field)
        if s.n == 0:
            return
        L = lb_filed._lattice()
        _capi.call("lbm_ibm_spread", ctypes.byref(L), ctypes.byref(s), stream_handle())

    def MultiDirectForcingLoop(self, sphere_field, lb_filed):
        """ibm.py:248-253"""
        sphere_field.reset_force()
        for _ in range(self.MDFIteration):
            self.InterpolateBodyVelocities(sphere_field=sphere_field, lb_filed=lb_filed)
            self.SpreadBodyForces(sphere_field=sphere_field, lb_filed=lb_filed)
