"""LBField and MacroscopicEngine (taichi_lbm/lbm.py in the reference).

Same names, constructor arguments and methods; every per-step method launches
its CUDA kernel through the C ABI on the current torch stream.
"""
import ctypes

import numpy as np
import torch

from . import _capi
from .fields import Field, MaskField, Scalar0D, alloc, round_up

# taichi_lbm/lbm.py:44-45
WEIGHTS = (np.array([4, 1, 1, 1, 1, 0.25, 0.25, 0.25, 0.25], np.float32) / np.float32(9.0))
C = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]],
             np.int32)
OPP = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6], np.int32)


def cuda_device(device=None):
    if not torch.cuda.is_available():
        raise RuntimeError("taichi_lbm (GB300 build) needs a CUDA device; there is no CPU path")
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    d = torch.device(device)
    if d.type != "cuda":
        raise RuntimeError(f"device {d} is not a CUDA device")
    return d


def stream_handle():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class NeighborView:
    """LBField.neighbor (lbm.py:50) decoded from the bit form on demand:
    (NX, NY, 9, 2) int32, -1 where the link has no source."""

    def __init__(self, lb):
        self._lb = lb

    def to_numpy(self):
        lb = self._lb
        links = lb._links[:, :lb.NX].cpu().numpy().astype(np.int64).T & 0xFFFF
        i = np.arange(lb.NX)[:, None]
        j = np.arange(lb.NY)[None, :]
        out = np.zeros((lb.NX, lb.NY, 9, 2), np.int32)
        classified = (links & 0x8000) != 0
        for k in range(9):
            ok = (links >> k) & 1
            out[:, :, k, 0] = np.where(classified, np.where(ok == 1, i - C[k, 0], -1), 0)
            out[:, :, k, 1] = np.where(classified, np.where(ok == 1, j - C[k, 1], -1), 0)
        return out

    def __getitem__(self, key):
        return self.to_numpy()[key]


class LBField:
    """Lattice state of one D2Q9 simulation (taichi_lbm/lbm.py:5-142).

    num_components > 1 (up to 4) keeps one set of populations, density,
    pressure, psi, Shan-Chen force and body force per component (the
    component-major LbmMCLattice layout) beside the mixture fields; such a
    lattice runs the per-stage multi-component kernels (MacroscopicEngine,
    ShanChenForceC2, BGKCollision, PeriodicAllBoundary, PeriodicPsi_LR/BT).
    """

    def __init__(self, name, NX, NY, num_components, device=None):
        nc = int(num_components)
        if not 1 <= nc <= _capi.MC_MAX:
            raise ValueError(f"num_components must be 1..{_capi.MC_MAX}")
        dev = cuda_device(device)
        self.device = dev
        self.name = name
        self.NX, self.NY = int(NX), int(NY)
        self.nc = nc
        self.num_components = Scalar0D(nc)
        self.pitch = round_up(self.NX, 32)
        self.psi_pitch = round_up(self.NX + 2, 32)
        nx, ny, P = self.NX, self.NY, self.pitch
        lead = (nc,) if nc > 1 else ()  # per-component arrays: a leading component axis
        self._f = alloc(lead + (9, ny, P), dev)
        self._f2 = alloc(lead + (9, ny, P), dev)
        self._rho = alloc(lead + (ny, P), dev)
        self._total_rho = alloc((ny, P), dev)
        self._pressure = alloc(lead + (ny, P), dev)
        self._total_pressure = alloc((ny, P), dev)
        self._shear_rate = alloc(lead + (ny, P), dev)
        self._T = alloc((ny, P), dev)
        self._vel = alloc((2, ny, P), dev)
        self._body_force = alloc(lead + (2, ny, P), dev)
        self._SCforce = alloc(lead + (2, ny, P), dev)
        self._psi = alloc(lead + (ny + 2, self.psi_pitch), dev)
        self._mask_dev = alloc((ny, P), dev, torch.int32)
        self._links = alloc((ny, P), dev, torch.int16)
        self._mask_version = -1

        self.f = Field(self, "_f", nx, ny, "vc", 9, nc=nc)
        self.f2 = Field(self, "_f2", nx, ny, "vc", 9, nc=nc)
        self.rho = Field(self, "_rho", nx, ny, "sc", nc=nc)
        self.pressure = Field(self, "_pressure", nx, ny, "sc", nc=nc)
        self.body_force = Field(self, "_body_force", nx, ny, "vc", 2, nc=nc)
        self.shear_rate = Field(self, "_shear_rate", nx, ny, "sc", nc=nc)
        self.SCforce = Field(self, "_SCforce", nx, ny, "vc", 2, nc=nc)
        self.vel = Field(self, "_vel", nx, ny, "v", 2)
        self.total_rho = Field(self, "_total_rho", nx, ny, "s")
        self.total_pressure = Field(self, "_total_pressure", nx, ny, "s")
        self.T = Field(self, "_T", nx, ny, "s")
        self.mask = MaskField(nx, ny)
        self.neighbor = NeighborView(self)
        self.time = Scalar0D(0)

        self.NPOP = 9
        self.weights = WEIGHTS.copy()
        self.c = C.copy()
        self.gravity_force = np.zeros(2, np.float32)
        self.sc_field = None
        # unit conversion (lbm.py:58-104)
        self.Ct = self.Cl = self.C_rho = self.Cu = self.C_pressure = 1.0
        self.C_force = self.C_torque = self.C_temperature = self.Cnu = self.C_T = 1.0
        self.shear_viscosity_LB = np.zeros(1, np.float32)
        self.bulk_viscosity_LB = np.zeros(1, np.float32)
        self._init_snapshot = None
        self.keep_init_snapshot = False
        self._fused_owner = None

    # ------------------------------------------------------------ plumbing
    def _sync_mask(self):
        if self._mask_version != self.mask.version:
            m = torch.as_tensor(self.mask.arr.T.copy(), device=self.device)
            self._mask_dev[:, :self.NX].copy_(m)
            self._mask_version = self.mask.version

    def _lattice(self, geometry_only=False):
        """The LbmLattice struct for the current buffers (geometry_only: just
        the mask and link table, for any number of components)."""
        if self.nc > 1 and geometry_only:
            self._sync_mask()
            L = _capi.LbmLattice()
            L.nx, L.ny, L.pitch, L.psi_pitch = self.NX, self.NY, self.pitch, self.psi_pitch
            L.mask = self._mask_dev.data_ptr()
            L.links = self._links.data_ptr()
            return L
        if self.nc > 1:
            raise NotImplementedError("this operation runs on single-component lattices; a "
                                      f"{self.nc}-component lattice runs the multi-component kernels")
        self._sync_mask()
        L = _capi.LbmLattice()
        L.nx, L.ny, L.pitch, L.psi_pitch = self.NX, self.NY, self.pitch, self.psi_pitch
        for name in ("f", "f2", "rho", "total_rho", "pressure", "total_pressure", "shear_rate",
                     "vel", "body_force", "psi"):
            setattr(L, name, getattr(self, "_" + name).data_ptr())
        L.temperature = self._T.data_ptr()
        L.sc_force = self._SCforce.data_ptr()
        L.mask = self._mask_dev.data_ptr()
        L.links = self._links.data_ptr()
        g = np.asarray(self.gravity_force, np.float32).reshape(2)
        L.gravity[0], L.gravity[1] = float(g[0]), float(g[1])
        return L

    def _mclattice(self):
        """The LbmMCLattice struct (every component) for the current buffers."""
        L = _capi.LbmMCLattice()
        L.nx, L.ny, L.pitch, L.psi_pitch, L.nc = self.NX, self.NY, self.pitch, self.psi_pitch, self.nc
        for name in ("f", "f2", "rho", "total_rho", "pressure", "total_pressure", "vel", "body_force", "psi"):
            setattr(L, name, getattr(self, "_" + name).data_ptr())
        L.temperature = self._T.data_ptr()
        L.sc_force = self._SCforce.data_ptr()
        g = np.asarray(self.gravity_force, np.float32).reshape(2)
        L.gravity[0], L.gravity[1] = float(g[0]), float(g[1])
        return L

    def _sync_fused(self):
        """Bring f/f2/moments up to date if a fused solver holds newer state."""
        if self._fused_owner is not None:
            self._fused_owner.sync()

    # ------------------------------------------------------------ API
    def init_conversion(self, params):
        """lbm.py:58-76 (unit conversion factors)."""
        p = {"Cl": None, "Ct": None, "C_rho": None, "C_pressure": None, "C_temperature": None}
        p.update(params)
        self.Ct, self.Cl = p["Ct"], p["Cl"]
        self.Cu = self.Cl / self.Ct
        self.Cnu = self.Cl ** 2 / self.Ct
        self.C_rho, self.C_pressure, self.C_temperature = p["C_rho"], p["C_pressure"], p["C_temperature"]
        self.C_force = self.Cl ** 3 * self.C_rho / self.Ct ** 2
        self.C_torque = self.C_force * self.Cl

    def set_gravity(self, g):
        self.gravity_force = np.asarray(g, np.float32).reshape(2)

    def get_Cforce(self):
        return self.C_force

    def get_Ctorque(self):
        return self.C_torque

    def get_Cu(self):
        return self.Cu

    def init_LBM(self, collsion, group):
        """f = f2 = feq(rho, vel) over the group (lbm.py:119-125)."""
        self._sync_fused()
        if self.keep_init_snapshot:  # host copy of the initial moments, for case descriptions
            self._init_snapshot = (self.rho.to_numpy()[:, :, 0].copy(), self.vel.to_numpy().copy(),
                                   self.T.to_numpy().copy())
        if self.nc > 1:
            L = self._mclattice()
            _capi.call("lbm_mc_init_feq", ctypes.byref(L), group.on(self).ptr, group.n, stream_handle())
            return
        L = self._lattice()
        _capi.call("lbm_init_feq", ctypes.byref(L), group.on(self).ptr, group.n, stream_handle())

    def neighbor_classify(self):
        """Pull-source table from the mask (lbm.py:127-142)."""
        L = self._lattice(geometry_only=True)
        _capi.call("lbm_neighbor_classify", ctypes.byref(L), stream_handle())

    def links_host(self):
        return (self._links[:, :self.NX].cpu().numpy().astype(np.int64).T & 0xFFFF).astype(np.int32)


class MacroscopicEngine:
    """Moment stage of the step (taichi_lbm/lbm.py:145-237)."""

    def __init__(self, group):
        self.group = group

    def time_updata(self, lb_field):
        lb_field.time[None] = lb_field.time[None] + 1

    def _mc(self, fn, lb_field, *extra):
        L = lb_field._mclattice()
        _capi.call(fn, ctypes.byref(L), *extra, self.group.on(lb_field).ptr, self.group.n, stream_handle())

    def density(self, lb_field):
        if lb_field.nc > 1:
            return self._mc("lbm_mc_density", lb_field)
        lb_field._sync_fused()
        L = lb_field._lattice()
        _capi.call("lbm_density", ctypes.byref(L), self.group.on(lb_field).ptr, self.group.n, stream_handle())

    def pressure(self, lb_field):
        if lb_field.nc > 1:  # pressure2 (lbm.py:185-202)
            sc = lb_field.sc_field
            if sc is None or not hasattr(sc, "mc_struct"):
                raise NotImplementedError("a multi-component lattice's pressure needs ShanChenForceC2")
            return self._mc("lbm_mc_pressure2", lb_field, ctypes.byref(sc.mc_struct()))
        lb_field._sync_fused()
        L = lb_field._lattice()
        sc = lb_field.sc_field
        _capi.call("lbm_pressure", ctypes.byref(L), self.group.on(lb_field).ptr, self.group.n,
                   0 if sc is None else 1, 0.0 if sc is None else float(sc.g_coh), stream_handle())

    pressure0 = pressure
    pressure1 = pressure
    pressure2 = pressure

    def force_density(self, lb_field):
        if lb_field.nc > 1:
            return self._mc("lbm_mc_force_density", lb_field)
        lb_field._sync_fused()
        L = lb_field._lattice()
        _capi.call("lbm_force_density", ctypes.byref(L), self.group.on(lb_field).ptr, self.group.n,
                   stream_handle())

    def velocity(self, lb_field):
        if lb_field.nc > 1:
            return self._mc("lbm_mc_velocity", lb_field)
        lb_field._sync_fused()
        L = lb_field._lattice()
        _capi.call("lbm_velocity", ctypes.byref(L), self.group.on(lb_field).ptr, self.group.n, stream_handle())
