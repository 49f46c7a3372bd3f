"""Shan-Chen pseudopotential model: equations of state (taichi_lbm/EOS.py),
the single- and two-component forces (taichi_lbm/ExternalForce.py) and psi
boundaries (taichi_lbm/SCBoundaryCondition.py)."""
import ctypes

import numpy as np
import torch

from . import _capi
from .boundary import BoundaryCondition, PlaneBoundary, evaluate_predicate
from .fields import Field
from .lbm import WEIGHTS, C, stream_handle


class Pseudopotential:
    """EOS.py:5-38.  Like the reference, rho_cr, pressure_cr and
    temperature_cr are required keys."""

    kind = None

    def __init__(self, params):
        p = {"a": None, "b": None, "R": 1.0, "G": 1.0}
        p.update(params)
        self.params = dict(params)
        self.a, self.b, self.R, self.G = p["a"], p["b"], p["R"], p["G"]
        self.rho_cr = params["rho_cr"]
        self.pressure_cr = params["pressure_cr"]
        self.temperature_cr = params["temperature_cr"]
        self.omega = params.get("omega", 0.0)

    def EOS(self, dens, T):
        raise NotImplementedError

    def get_psi(self, dens, T):
        """Host evaluation in float32 (EOS.py:28-32)."""
        dens = np.asarray(dens, np.float32)
        T = np.asarray(T, np.float32)
        p = self.EOS(dens, T)
        return np.sqrt(np.abs(np.float32(6.0 / self.G) * (p - dens / np.float32(3.0))))

    def struct(self):
        e = _capi.LbmEos()
        e.kind = self.kind
        e.a, e.b = float(self.a or 0.0), float(self.b or 0.0)
        e.R, e.G = float(self.R), float(self.G)
        e.rho0 = 0.0
        e.omega = float(self.omega or 0.0)
        e.T_cr = float(self.temperature_cr or 1.0)
        return e


class SC_psi:
    """EOS.py:40-47"""

    kind = _capi.EOS_SC

    def __init__(self, rho0):
        self.rho0 = rho0

    def get_psi(self, dens, T):
        d = np.asarray(dens, np.float32)
        r0 = np.float32(self.rho0)
        return r0 * (np.float32(1) - np.exp(-d / r0))

    def struct(self):
        e = _capi.LbmEos()
        e.kind = self.kind
        e.rho0 = float(self.rho0)
        e.R = e.G = 1.0
        e.T_cr = 1.0
        return e


class vdW_psi(Pseudopotential):
    """EOS.py:50-58"""
    kind = _capi.EOS_VDW

    def EOS(self, dens, T):
        return dens * np.float32(self.R) * T / (1 - np.float32(self.b) * dens) - np.float32(self.a) * dens ** 2


class RK_psi(Pseudopotential):
    """EOS.py:61-69"""
    kind = _capi.EOS_RK

    def EOS(self, dens, T):
        a, b, R = (np.float32(v) for v in (self.a, self.b, self.R))
        return dens * R * T / (1 - b * dens) - a * dens ** 2 / np.sqrt(T) / (1 + b * dens)


class PR_psi(Pseudopotential):
    """EOS.py:72-82"""
    kind = _capi.EOS_PR

    def __init__(self, params):
        super().__init__(params)
        self.omega = params["omega"]

    def EOS(self, dens, T):
        a, b, R = (np.float32(v) for v in (self.a, self.b, self.R))
        om = self.omega
        kap = np.float32(0.37464 + 1.54226 * om - 0.269922 * om * om)
        alpha = (1 + kap * (1 - np.sqrt(T / np.float32(self.temperature_cr)))) ** 2
        return dens * R * T / (1 - b * dens) - a * alpha * dens ** 2 / (1 + 2 * b * dens - (b * dens) ** 2)


class CS_psi(Pseudopotential):
    """EOS.py:85-95 (Carnahan-Starling)"""
    kind = _capi.EOS_CS

    def EOS(self, dens, T):
        a, b, R = (np.float32(v) for v in (self.a, self.b, self.R))
        b4 = b * dens / 4
        return dens * R * T * (1 + b4 + b4 ** 2 - b4 ** 3) / (1 - b4) ** 3 - a * dens ** 2


class ShanChenModel:
    """ExternalForce.py:5-23: psi on a one-node halo around the lattice."""

    def __init__(self, lb_field, group):
        self.group = group
        self.wc = (WEIGHTS[:, None] * C).astype(np.float32)
        self.psi_field = Field(lb_field, "_psi", lb_field.NX, lb_field.NY, "sc", halo=1, nc=lb_field.nc)


class ShanChenForceC1(ShanChenModel):
    """ExternalForce.py:27-63: single-component Shan-Chen force."""

    def __init__(self, params):
        p = {"lb_field": None, "g_coh": None, "group": None, "psi": None}
        p.update(params)
        super().__init__(p["lb_field"], p["group"])
        self.g_coh = p["g_coh"]
        self.psi = p["psi"]

    def update_psi(self, lb_field):
        lb_field._sync_fused()
        L = lb_field._lattice()
        e = self.psi.struct()
        _capi.call("lbm_sc_update_psi", ctypes.byref(L), ctypes.byref(e), self.group.on(lb_field).ptr,
                   self.group.n, stream_handle())

    def cau_SCforce(self, lb_field):
        lb_field._sync_fused()
        L = lb_field._lattice()
        _capi.call("lbm_sc_force", ctypes.byref(L), float(self.g_coh), self.group.on(lb_field).ptr,
                   self.group.n, stream_handle())


class ShanChenForceC2(ShanChenModel):
    """ExternalForce.py:66-117: two-component Shan-Chen force on a lattice
    with num_components = 2.  params: lb_field, g_coh (cohesion matrix,
    nc x nc), gadh (adhesion per component), group, psi_list (the two
    components' pseudopotentials) and fluid_strategy(x, y), a predicate that
    may be called on halo coordinates (-1..NX, -1..NY): cohesion acts from
    neighbours where it holds, adhesion from the others."""

    def __init__(self, params):
        p = {"lb_field": None, "g_coh": None, "gadh": None, "group": None, "psi_list": None,
             "fluid_strategy": None}
        p.update(params)
        lb = p["lb_field"]
        if lb.nc < 2:
            raise ValueError("ShanChenForceC2 needs a lattice with num_components >= 2")
        super().__init__(lb, p["group"])
        self.lb = lb
        self.g_coh = np.asarray(p["g_coh"], np.float32).reshape(lb.nc, lb.nc)
        self.g_adh = np.asarray(p["gadh"] if p["gadh"] is not None else np.zeros(lb.nc), np.float32).reshape(-1)
        self.psi1, self.psi2 = p["psi_list"][0], p["psi_list"][1]
        self.fluid_strategy = p["fluid_strategy"]
        fn = self.fluid_strategy or (lambda i, j: True)
        sel = evaluate_predicate(fn, lb.NX + 2, lb.NY + 2, -1, -1)
        fluid = np.zeros((lb.NY + 2, lb.psi_pitch), np.uint8)
        fluid[:, :lb.NX + 2] = sel.T
        self._fluid = torch.as_tensor(fluid, device=lb.device)

    def mc_struct(self):
        s = _capi.LbmMCShanChen()
        nc = self.lb.nc
        for a in range(nc):
            for b in range(nc):
                s.g_coh[a][b] = float(self.g_coh[a, b])
            s.g_adh[a] = float(self.g_adh[a]) if a < self.g_adh.size else 0.0
        s.eos[0] = self.psi1.struct()
        s.eos[1] = self.psi2.struct()
        s.fluid = self._fluid.data_ptr()
        return s

    def _call(self, fn, lb_field):
        L = lb_field._mclattice()
        _capi.call(fn, ctypes.byref(L), ctypes.byref(self.mc_struct()), self.group.on(lb_field).ptr,
                   self.group.n, stream_handle())

    def update_psi(self, lb_field):
        """ExternalForce.py:86-92"""
        self._call("lbm_mc_update_psi", lb_field)

    def cau_SCforce(self, lb_field):
        """ExternalForce.py:96-117"""
        self._call("lbm_mc_sc_force", lb_field)


# ------------------------------------------------------------ psi boundaries
def _psi_periodic(lb_field, axis):
    if lb_field.nc > 1:
        L = lb_field._mclattice()
        _capi.call("lbm_mc_psi_periodic", ctypes.byref(L), axis, stream_handle())
    else:
        L = lb_field._lattice()
        _capi.call("lbm_psi_periodic", ctypes.byref(L), axis, stream_handle())


class PeriodicPsi_LR:
    """SCBoundaryCondition.py:126-134 (every component)"""

    def apply(self, lb_field):
        _psi_periodic(lb_field, 0)


class PeriodicPsi_BT:
    """SCBoundaryCondition.py:136-144 (every component)"""

    def apply(self, lb_field):
        _psi_periodic(lb_field, 1)


class FixedPsi(BoundaryCondition):
    """SCBoundaryCondition.py:113-123"""

    def __init__(self, spec, psi_value):
        super().__init__(spec)
        self.psi_value = psi_value

    def apply(self, lb_field):
        L = lb_field._lattice()
        _capi.call("lbm_psi_fixed", ctypes.byref(L), self.group.on(lb_field, halo=1).ptr, self.group.n,
                   float(self.psi_value), stream_handle())


class OpenBoundaryPsi(PlaneBoundary):
    """SCBoundaryCondition.py:9-15: open boundaries of the psi field.  The
    group is classified over psi coordinates (halo allowed, e.g. with
    BoundaryClassifier((NX + 2, NY + 2), offset=(-1, -1))); each node is
    set from its neighbours x - c_direction and x - 2 c_direction."""

    psi_kind = None
    reads = 1  # psi neighbours read along -c_direction

    def apply(self, lb_field):
        g = self.group
        c = lb_field.c[self.direction]
        g.on(lb_field, halo=1)
        for d in range(1, self.reads + 1):  # the neighbours lie on the psi grid
            g.require_inside(lb_field.NX + 2, lb_field.NY + 2, (d * int(c[0]) - 1, d * int(c[1]) - 1),
                             what=type(self).__name__)
        if self.psi_kind in (_capi.PSI_OPEN_CONV1, _capi.PSI_OPEN_CONV2):  # and x - c inside the lattice
            g.require_inside(lb_field.NX, lb_field.NY, (int(c[0]), int(c[1])), what=type(self).__name__)
        L = lb_field._lattice()
        _capi.call("lbm_psi_open", ctypes.byref(L), g.ptr, g.n, self.psi_kind, int(self.direction),
                   stream_handle())


class OpenNeumannPsi(OpenBoundaryPsi):
    """SCBoundaryCondition.py:19-34: psi(x) = psi(x - c)."""
    psi_kind = _capi.PSI_OPEN_NEUMANN


class OpenConvective1orderPsi(OpenBoundaryPsi):
    """SCBoundaryCondition.py:36-61: psi(x) = (psi(x) + lambda psi(x - c)) /
    (1 + lambda), lambda = |u| averaged over the neighbours x - c."""
    psi_kind = _capi.PSI_OPEN_CONV1


class OpenConvective2orderPsi(OpenBoundaryPsi):
    """SCBoundaryCondition.py:64-91: the second-order convective form over
    x - c and x - 2c."""
    psi_kind = _capi.PSI_OPEN_CONV2
    reads = 2


class OpenExtrapolationPsi(OpenBoundaryPsi):
    """SCBoundaryCondition.py:94-110: psi(x) = 2 psi(x - c) - psi(x - 2c)."""
    psi_kind = _capi.PSI_OPEN_EXTRAP
    reads = 2


class BoundaryEngineSC:
    """SCBoundaryCondition.py:149-160"""

    def __init__(self):
        self.boundary_conditions = {}

    def add_boundary_condition(self, name, bc):
        self.boundary_conditions[name] = bc

    def apply_boundary_conditions(self, lb_field):
        for bc in self.boundary_conditions.values():
            bc.apply(lb_field)
