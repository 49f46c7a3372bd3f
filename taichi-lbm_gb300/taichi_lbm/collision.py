"""Collision operators (taichi_lbm/CollisionEngine.py) and rheology
(taichi_lbm/FluidModels.py).

Same classes, parameter dictionaries and methods; ``initTau``,
``shear_rate``, ``relaxation_time`` and ``apply`` launch CUDA kernels.
Extension keys (absent from the reference): ``mrt_s`` (9 MRT relaxation
rates written over ``diag`` for the group after ``initTau``) and
``tau_clamp`` ((tau_min, tau_max), applied before ``initTau``).
"""
import ctypes

import numpy as np
import torch

from . import _capi
from .fields import Field, alloc, round_up
from .lbm import C, WEIGHTS, stream_handle

# CollisionEngine.py:273-282
MRT_M = np.array([
    [1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0],
    [-4.0, -1.0, -1.0, -1.0, -1.0, 2.0, 2.0, 2.0, 2.0],
    [4.0, -2.0, -2.0, -2.0, -2.0, 1.0, 1.0, 1.0, 1.0],
    [0.0, 1.0, 0.0, -1.0, 0.0, 1.0, -1.0, -1.0, 1.0],
    [0.0, -2.0, 0.0, 2.0, 0.0, 1.0, -1.0, -1.0, 1.0],
    [0.0, 0.0, 1.0, 0.0, -1.0, 1.0, 1.0, -1.0, -1.0],
    [0.0, 0.0, -2.0, 0.0, 2.0, 1.0, 1.0, -1.0, -1.0],
    [0.0, 1.0, -1.0, 1.0, -1.0, 0.0, 0.0, 0.0, 0.0],
    [0.0, 0.0, 0.0, 0.0, 0.0, 1.0, -1.0, 1.0, -1.0]])


def feq_numpy(vel, rho):
    """Equilibrium populations (CollisionEngine.py:15-18), float32."""
    vel = np.asarray(vel, np.float32)
    eu = C.astype(np.float32) @ vel
    uv = np.float32(vel[0] * vel[0] + vel[1] * vel[1])
    return WEIGHTS * np.float32(rho) * (1 + 3 * eu + np.float32(4.5) * eu * eu - np.float32(1.5) * uv)


class NewtonianFluid:
    """FluidModels.py:9-17"""

    def __init__(self, nu):
        self.nu = nu

    def apparent_viscosity(self, shear_rate, rho):
        return self.nu


class PowerLawFluid:
    """FluidModels.py:20-29"""

    def __init__(self, m, n):
        self.m = m
        self.n = n

    def apparent_viscosity(self, shear_rate, rho):
        return self.m * np.asarray(shear_rate, np.float32) ** np.float32(self.n - 1.0)


class Collision:
    """CollisionEngine.py:6-34"""

    model = None

    def __init__(self, group, fluid_model):
        self.group = group
        self.fluid_model = fluid_model
        self.tau_min = 0.5000001
        self.tau_max = 4.0

    def f_eq(self, c, w, vel, rho):
        return feq_numpy(vel, rho)

    def f_force(self, c, w, F, vel):
        F = np.asarray(F, np.float32)
        vel = np.asarray(vel, np.float32)
        cF = C.astype(np.float32) @ F
        cu = C.astype(np.float32) @ vel
        uF = np.float32(vel[0] * F[0] + vel[1] * F[1])
        return WEIGHTS * (3 * cF + 9 * cF * cu - 3 * uF)

    def tau_max_min(self, tau):
        return min(max(tau, self.tau_min), self.tau_max)

    def _setup(self, params):
        p = dict(params)
        self.NX, self.NY = int(p["NX"]), int(p["NY"])
        self.nc = int(p.get("num_components") or 1)
        if self.nc != 1 and self.model != _capi.BGK:
            raise NotImplementedError("multi-component lattices collide with BGKCollision in this build")
        self.pitch = round_up(self.NX, 32)
        self.device = self.group.group.device
        self.nu = np.asarray(p["shearviscosity"], np.float32).reshape(-1)[:max(1, self.nc)]
        clamp = p.get("tau_clamp")
        if clamp is not None:
            self.tau_min, self.tau_max = float(clamp[0]), float(clamp[1])

    def _fm(self):
        fm = self.fluid_model
        if isinstance(fm, PowerLawFluid):
            return _capi.POWERLAW, float(fm.m), float(fm.n)
        return _capi.NEWTONIAN, 0.0, 1.0

    def _struct(self):
        c = _capi.LbmCollision()
        c.model = self.model
        kind, m, n = self._fm()
        c.fluid_model = kind
        fm_nu = getattr(self.fluid_model, "nu", None)
        c.nu = float(fm_nu if (kind == _capi.NEWTONIAN and fm_nu is not None) else self.nu[0])
        c.nu_bulk = float(getattr(self, "nu_bulk", np.zeros(1))[0])
        c.magic = float(getattr(self, "magic", np.zeros(1))[0])
        c.tau_min, c.tau_max = float(self.tau_min), float(self.tau_max)
        c.pl_m, c.pl_n = m, n
        for name in ("tau", "tau_sym", "tau_antisym", "diag"):
            t = getattr(self, "_" + name, None)
            setattr(c, name, None if t is None else t.data_ptr())
        minv = getattr(self, "M_inverse", None)
        if minv is not None:
            for q, v in enumerate(np.asarray(minv, np.float32).reshape(81)):
                c.m_inverse[q] = float(v)
        return c

    def _init_struct(self):
        c = self._struct()
        c.nu = float(self.nu[0])
        return c

    def _call(self, fn, lb_field, init=False):
        if lb_field.nc > 1:
            if fn != "lbm_collision_apply":
                raise NotImplementedError("multi-component lattices: BGK collision with Newtonian "
                                          "components only (no local relaxation)")
            L = lb_field._mclattice()
            _capi.call("lbm_mc_bgk_apply", ctypes.byref(L), ctypes.c_void_p(self._tau.data_ptr()),
                       self.group.on(lb_field).ptr, self.group.n, stream_handle())
            return
        lb_field._sync_fused()
        L = lb_field._lattice()
        c = self._init_struct() if init else self._struct()
        _capi.call(fn, ctypes.byref(L), ctypes.byref(c), self.group.on(lb_field).ptr, self.group.n,
                   stream_handle())

    def initTau(self, lb_field=None):
        c = self._init_struct()
        L = _capi.LbmLattice()
        L.nx, L.ny, L.pitch = self.NX, self.NY, self.pitch
        _capi.call("lbm_collision_init_tau", ctypes.byref(L), ctypes.byref(c), self.group.on(self).ptr,
                   self.group.n, stream_handle())

    def shear_rate(self, lb_field):
        self._call("lbm_collision_shear_rate", lb_field)

    def relaxation_time(self, lb_field):
        self._call("lbm_collision_relaxation_time", lb_field)

    def apply(self, lb_field):
        self._call("lbm_collision_apply", lb_field)


class BGKCollision(Collision):
    """CollisionEngine.py:36-110"""

    model = _capi.BGK

    def __init__(self, params):
        p = {"group": None, "fluid_model": None, "NX": None, "NY": None, "num_components": None,
             "shearviscosity": None}
        p.update(params)
        super().__init__(p["group"], p["fluid_model"])
        self._setup(p)
        if self.nc > 1:
            # one relaxation time per component: tau = 3 nu_c + 1/2 on the
            # group (CollisionEngine.py:65-70), in float32 as the reference
            self._tau = alloc((self.nc, self.NY, self.pitch), self.device)
            self.tau = Field(self, "_tau", self.NX, self.NY, "sc", nc=self.nc)
            nd = torch.as_tensor(self.group.nodes, device=self.device).long()
            for c in range(self.nc):
                t = torch.tensor(float(self.nu[c]), dtype=torch.float32) * 3.0 + 0.5
                self._tau[c][nd[:, 1], nd[:, 0]] = t.to(self.device)
            return
        self._tau = alloc((self.NY, self.pitch), self.device)
        self.tau = Field(self, "_tau", self.NX, self.NY, "sc")
        self.initTau()


class TRTCollision(Collision):
    """CollisionEngine.py:113-245"""

    model = _capi.TRT

    def __init__(self, params):
        p = {"group": None, "fluid_model": None, "NX": None, "NY": None, "num_components": None,
             "shearviscosity": None, "magic": None}
        p.update(params)
        super().__init__(p["group"], p["fluid_model"])
        self._setup(p)
        self.magic = np.asarray(p["magic"], np.float32).reshape(-1)[:1]
        self._tau_sym = alloc((self.NY, self.pitch), self.device)
        self._tau_antisym = alloc((self.NY, self.pitch), self.device)
        self.tau_sym = Field(self, "_tau_sym", self.NX, self.NY, "sc")
        self.tau_antisym = Field(self, "_tau_antisym", self.NX, self.NY, "sc")
        self.initTau()


class MRTCollision(Collision):
    """CollisionEngine.py:247-451"""

    model = _capi.MRT

    def __init__(self, params):
        p = {"group": None, "fluid_model": None, "NX": None, "NY": None, "num_components": None,
             "shearviscosity": None, "bulkviscosity": None}
        p.update(params)
        super().__init__(p["group"], p["fluid_model"])
        self._setup(p)
        self.M = MRT_M.astype(np.float32)
        self.M_inverse = np.linalg.inv(MRT_M).astype(np.float32)
        self.nu_bulk = np.asarray(p["bulkviscosity"], np.float32).reshape(-1)[:1]
        self._diag = alloc((9, self.NY, self.pitch), self.device)
        self.diag = Field(self, "_diag", self.NX, self.NY, "vc", 9)
        self.initTau()
        if p.get("mrt_s") is not None:
            self.set_rates(p["mrt_s"])

    def set_rates(self, s):
        """Write the 9 relaxation rates over diag for every group node."""
        s = np.asarray(s, np.float32).reshape(9)
        nd = torch.as_tensor(self.group.nodes, device=self.device).long()
        for a in range(9):
            self._diag[a, nd[:, 1], nd[:, 0]] = float(s[a])


class HuangMRTCollision(MRTCollision):
    """CollisionEngine.py:453-515.  The reference class cannot be constructed
    (it calls MRTCollision.__init__ with positional arguments MRTCollision
    does not take), so there is no behaviour to reproduce."""

    def __init__(self, *args, **kwargs):
        raise NotImplementedError("HuangMRTCollision is not constructible in taichi-lbm either "
                                  "(CollisionEngine.py:455-456 passes arguments MRTCollision "
                                  "does not accept)")
