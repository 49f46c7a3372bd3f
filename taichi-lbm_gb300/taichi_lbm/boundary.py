"""Boundary grouping and boundary conditions (taichi_lbm/BoundaryCondition.py).

Grouping (MaskAndGroup / BoundarySpec / BoundaryClassifier) is setup work and
runs on the host: a geometry predicate is evaluated over the whole index box
(vectorised over numpy index arrays when the predicate allows it, node by node
otherwise) and the selected nodes are uploaded as an int32 (i, j) list.  The
reference appends nodes with an atomic counter, so its order is arbitrary;
here nodes are in memory order (j, then i) so that per-group kernels read
and write consecutive addresses.  Every per-step operation is a
CUDA kernel launched through the C ABI.
"""
import ctypes

import numpy as np
import torch

from . import _capi
from .lbm import stream_handle


class MaskAndGroup:
    """Node list of one boundary group (BoundaryCondition.py:8-12)."""

    def __init__(self, nodes, device):
        nodes = np.ascontiguousarray(np.asarray(nodes, np.int32).reshape(-1, 2))
        self.nodes = nodes
        self._checked = set()
        self.count = _Count(nodes.shape[0])
        self.group = torch.as_tensor(nodes if nodes.size else np.zeros((1, 2), np.int32),
                                     device=device)

    @property
    def n(self):
        return int(self.nodes.shape[0])

    @property
    def ptr(self):
        return ctypes.c_void_p(self.group.data_ptr())

    def on(self, lattice, halo=0):
        """Validate against a lattice (anything with NX, NY; halo=1 admits the
        psi ring) and return self."""
        self.require_inside(lattice.NX + 2 * halo, lattice.NY + 2 * halo, (-halo, -halo))
        return self

    def require_inside(self, nx, ny, shift=(0, 0), what="group"):
        """Raise unless every node (minus shift) lies in the lattice: the
        kernels index fields with these coordinates."""
        key = (nx, ny, tuple(shift))
        if key in self._checked:
            return
        nd = self.nodes - np.asarray(shift, np.int32)
        if nd.size and ((nd[:, 0] < 0).any() or (nd[:, 0] >= nx).any() or (nd[:, 1] < 0).any()
                        or (nd[:, 1] >= ny).any()):
            raise ValueError(f"{what} has nodes whose {'neighbour ' if any(shift) else ''}"
                             f"coordinates fall outside the {nx} x {ny} lattice")
        self._checked.add(key)


class _Count:
    def __init__(self, n):
        self.n = n

    def __getitem__(self, key):
        return self.n

    def __int__(self):
        return self.n


class BoundarySpec:
    """How boundary nodes are identified (BoundaryCondition.py:14-20).

    ``geometry_fn(i, j)`` selects nodes.  ``value_fn(i, j) -> (ux, uy)`` gives a
    per-node velocity to velocity boundaries (the reference stores value_fn but
    never reads it; here it is used, and a constant velocity_value remains the
    reference behaviour).  ``vectorized=False`` forces node-by-node evaluation.
    """

    def __init__(self, geometry_fn, direction=None, value_fn=None, vectorized=None):
        self.geometry_fn = geometry_fn
        self.direction = direction
        self.value_fn = value_fn
        self.vectorized = vectorized


_GRIDS = {}


def _index_grid(nx, ny, ox, oy):
    """(I, J) index arrays of the box, cached for the last few shapes."""
    key = (nx, ny, ox, oy)
    g = _GRIDS.get(key)
    if g is None:
        if len(_GRIDS) >= 4:
            _GRIDS.pop(next(iter(_GRIDS)))
        g = np.meshgrid(np.arange(nx) + ox, np.arange(ny) + oy, indexing="ij")
        for a in g:
            a.setflags(write=False)
        _GRIDS[key] = g
    return g


def evaluate_predicate(fn, nx, ny, ox=0, oy=0, vectorized=None):
    """Boolean (nx, ny) array of fn over the index box starting at (ox, oy)."""
    if vectorized is not False:
        I, J = _index_grid(nx, ny, ox, oy)
        try:
            r = np.asarray(fn(I, J))
            if r.shape == I.shape:
                return r.astype(bool)
        except Exception:
            if vectorized:
                raise
    out = np.zeros((nx, ny), bool)
    for i in range(nx):
        for j in range(ny):
            out[i, j] = bool(fn(i + ox, j + oy))
    return out


def evaluate_values(fn, nodes):
    """Per-node (n, 2) float32 values of value_fn."""
    if nodes.shape[0] == 0:
        return np.zeros((0, 2), np.float32)
    try:
        r = fn(nodes[:, 0], nodes[:, 1])
        a = np.asarray(r, np.float64)
        if a.shape == (2, nodes.shape[0]):
            return a.T.astype(np.float32).copy()
        if a.shape == (nodes.shape[0], 2):
            return a.astype(np.float32)
    except Exception:
        pass
    return np.array([np.asarray(fn(int(i), int(j)), np.float64).reshape(2) for i, j in nodes],
                    np.float32)


class BoundaryClassifier:
    """Builds node groups from specs (BoundaryCondition.py:22-39).

    ``shape`` is anything with a 2-D ``.shape`` (an LBField field, a numpy
    array) or a (NX, NY) tuple; ``offset`` shifts the index box (the reference
    uses a field with offset (-1, -1) for psi halos).
    """

    def __init__(self, shape, offset=None, device=None):
        if hasattr(shape, "shape") and not isinstance(shape, tuple):
            shp = tuple(shape.shape)[:2]
            offset = offset if offset is not None else getattr(shape, "offset", None)
        else:
            shp = tuple(shape)
        self.shape = shp
        self.offset = tuple(offset) if offset is not None else (0, 0)
        self.device = device

    def get_group(self, spec):
        sel = evaluate_predicate(spec.geometry_fn, self.shape[0], self.shape[1], self.offset[0],
                                 self.offset[1], spec.vectorized)
        # memory order (j, then i): consecutive group entries are consecutive
        # addresses, so the per-group kernels' accesses coalesce
        nodes = np.argwhere(sel.T)[:, ::-1].astype(np.int32) + np.asarray(self.offset, np.int32)
        dev = self.device
        if dev is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        return MaskAndGroup(nodes, dev)


class BoundaryCondition:
    """Base class (BoundaryCondition.py:41-54); kind LBM_BC_FLUID is a no-op."""

    kind = _capi.BC_FLUID

    def __init__(self, spec):
        self.spec = spec
        self.group = None
        self._per_node = None

    def precompute(self, classifier):
        self.group = classifier.get_group(self.spec)
        self._per_node = None

    def _struct(self, lb_field):
        b = _capi.LbmBoundary()
        b.kind = self.kind
        b.direction = int(getattr(self, "direction", 0) or 0)
        b.rho_value = float(getattr(self, "rho_value", 0.0) or 0.0)
        vel = self.velocity_array()
        b.velocity[0], b.velocity[1] = float(vel[0]), float(vel[1])
        pn = self.per_node_velocity()
        b.velocity_per_node = None if pn is None else pn.data_ptr()
        sc = lb_field.sc_field
        if sc is not None:
            b.g_coh = float(sc.g_coh)
            b.eos = sc.psi.struct()
        return b

    def velocity_array(self):
        v = getattr(self, "velocity_value", None)
        if v is None:
            return np.zeros(2, np.float32)
        return np.asarray(v, np.float32).reshape(2)

    def per_node_velocity(self):
        """(n, 2) device tensor when the spec carries a value_fn, else None."""
        fn = getattr(self.spec, "value_fn", None)
        if fn is None or not hasattr(self, "velocity_value"):
            return None
        if self._per_node is None:
            vals = evaluate_values(fn, self.group.nodes)
            self._per_node = torch.as_tensor(vals if vals.size else np.zeros((1, 2), np.float32),
                                             device=self.group.group.device)
        return self._per_node

    def per_node_velocity_host(self):
        fn = getattr(self.spec, "value_fn", None)
        if fn is None:
            return np.tile(self.velocity_array(), (self.group.n, 1))
        return evaluate_values(fn, self.group.nodes)

    # kinds that read the neighbour x - c_dir (1) or also x - 2 c_dir (2)
    NEIGHBOUR_DEPTH = {_capi.BC_VELOCITY_NEEM: 1, _capi.BC_PRESSURE_ABC: 1,
                       _capi.BC_PRESSURE_NEEM: 1, _capi.BC_OPEN_NEUMANN: 1, _capi.BC_OPEN_CONV1: 1,
                       _capi.BC_OPEN_CONV2: 2, _capi.BC_OPEN_EXTRAP: 2}

    def check(self, lb_field):
        g = self.group
        g.require_inside(lb_field.NX, lb_field.NY, what=type(self).__name__)
        depth = self.NEIGHBOUR_DEPTH.get(self.kind, 0)
        if depth:
            c = lb_field.c[self.direction]
            for d in range(1, depth + 1):
                g.require_inside(lb_field.NX, lb_field.NY, (d * int(c[0]), d * int(c[1])),
                                 what=type(self).__name__)

    def apply(self, lb_field):
        if self.kind == _capi.BC_FLUID:
            return
        if lb_field.nc > 1:
            if self.kind != _capi.BC_PERIODIC:
                raise NotImplementedError(f"{type(self).__name__} on a multi-component lattice: only "
                                          "PeriodicAllBoundary streams every component in this build")
            self.group.require_inside(lb_field.NX, lb_field.NY, what=type(self).__name__)
            L = lb_field._mclattice()
            _capi.call("lbm_mc_stream_periodic", ctypes.byref(L), self.group.ptr, self.group.n,
                       stream_handle())
            return
        self.check(lb_field)
        lb_field._sync_fused()
        L = lb_field._lattice()
        b = self._struct(lb_field)
        _capi.call("lbm_boundary_apply", ctypes.byref(L), ctypes.byref(b), self.group.ptr,
                   self.group.n, stream_handle())


class PlaneBoundary(BoundaryCondition):
    """BoundaryCondition.py:57-72; direction 1..4 picks the unknown populations."""

    UNKNOWN = {1: [3, 6, 7], 3: [1, 5, 8], 4: [2, 5, 6], 2: [4, 7, 8], None: None}

    def __init__(self, spec, direction):
        super().__init__(spec)
        self.direction = direction
        self.unknow = self.UNKNOWN[direction]


class VelocityBoundary(PlaneBoundary):
    def __init__(self, spec, velocity_value, direction):
        super().__init__(spec, direction)
        self.velocity_value = velocity_value


class VelocityBB(VelocityBoundary):
    """BoundaryCondition.py:80-102"""
    kind = _capi.BC_VELOCITY_BB


class NEEMMethod:
    """BoundaryCondition.py:104-129 (host restatement for inspection)."""

    @staticmethod
    def f_eq(c, w, vel, rho):
        from .collision import feq_numpy
        return feq_numpy(vel, rho)


class VelocityEquilibrium(VelocityBoundary, NEEMMethod):
    """BoundaryCondition.py:132-147"""
    kind = _capi.BC_VELOCITY_EQ


class VelocityNEEM(VelocityBoundary, NEEMMethod):
    """BoundaryCondition.py:149-166"""
    kind = _capi.BC_VELOCITY_NEEM


class PressureBoundary(PlaneBoundary):
    def __init__(self, spec, rho_value, direction):
        super().__init__(spec, direction)
        self.rho_value = rho_value


class PressureABC(PressureBoundary):
    """BoundaryCondition.py:177-205"""
    kind = _capi.BC_PRESSURE_ABC


class PressureNEEM(PressureBoundary, NEEMMethod):
    """BoundaryCondition.py:209-226 (rho_value reaches total_rho only, as in the reference)."""
    kind = _capi.BC_PRESSURE_NEEM


class BounceBackWall(BoundaryCondition):
    """BoundaryCondition.py:231-259"""
    kind = _capi.BC_BOUNCEBACK

    def __init__(self, spec):
        super().__init__(spec)
        self.bounce_map = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6], np.int32)


class OpenBoundary(PlaneBoundary):
    pass


class OpenNeumann(OpenBoundary):
    """BoundaryCondition.py:315-334"""
    kind = _capi.BC_OPEN_NEUMANN


class OpenConvective1order(OpenBoundary):
    """BoundaryCondition.py:337-359"""
    kind = _capi.BC_OPEN_CONV1


class OpenConvective2order(OpenBoundary):
    """BoundaryCondition.py:362-390 (needs lb_field.sc_field)"""
    kind = _capi.BC_OPEN_CONV2

    def apply(self, lb_field):
        if lb_field.sc_field is None:
            raise RuntimeError("OpenConvective2order needs a Shan-Chen field (lb_field.sc_field)")
        super().apply(lb_field)


class OpenExtrapolation(OpenBoundary):
    """BoundaryCondition.py:394-411"""
    kind = _capi.BC_OPEN_EXTRAP


class PeriodicAllBoundary(BoundaryCondition):
    """BoundaryCondition.py:419-432"""
    kind = _capi.BC_PERIODIC


class InsideBoundary(BoundaryCondition):
    """BoundaryCondition.py:435-449"""
    kind = _capi.BC_INSIDE


class FluidBoundary(BoundaryCondition):
    """BoundaryCondition.py:452-455"""
    kind = _capi.BC_FLUID


STREAM_KINDS = (_capi.BC_PERIODIC, _capi.BC_INSIDE, _capi.BC_BOUNCEBACK)


class BoundaryEngine:
    """Ordered boundary conditions plus mask helpers (BoundaryCondition.py:459-510)."""

    def __init__(self):
        self.boundary_conditions = {}

    def Mask_rectangle_identify(self, lb_field, xmin, xmax, ymin, ymax):
        """Open rectangle -> mask -1, in the reference's f32 arithmetic (:464-469)."""
        i = np.arange(lb_field.NX)[:, None]
        j = np.arange(lb_field.NY)[None, :]
        xmin, xmax, ymin, ymax = (np.float32(v) for v in (xmin, xmax, ymin, ymax))
        sel = (i < xmax) & (i > xmin) & (j < ymax) & (j > ymin)
        m = lb_field.mask.to_numpy()
        m[sel] = -1
        lb_field.mask.from_numpy(m)

    def Mask_cricle_identify(self, lb_field, x, y, r):
        """Strict disc -> mask -1, in the reference's f32 arithmetic (:471-475)."""
        x, y, r = np.float32(x), np.float32(y), np.float32(r)
        dx = np.arange(lb_field.NX, dtype=np.float32)[:, None] - x
        dy = np.arange(lb_field.NY, dtype=np.float32)[None, :] - y
        sel = (dx * dx + dy * dy) < (r * r)
        m = lb_field.mask.to_numpy()
        m[sel] = -1
        lb_field.mask.from_numpy(m)

    Mask_circle_identify = Mask_cricle_identify

    def add_boundary_condition(self, name, bc):
        self.boundary_conditions[name] = bc

    def apply_boundary_conditions(self, lb_field):
        for bc in self.boundary_conditions.values():
            bc.apply(lb_field)

    def group_map(self, lb_field):
        """(NX, NY) int16: 1-based index of the last boundary covering each node."""
        img = np.zeros((lb_field.NX, lb_field.NY), np.int16)
        for n, bc in enumerate(self.boundary_conditions.values(), 1):
            nd = bc.group.nodes
            ok = (nd[:, 0] >= 0) & (nd[:, 0] < lb_field.NX) & (nd[:, 1] >= 0) & (nd[:, 1] < lb_field.NY)
            img[nd[ok, 0], nd[ok, 1]] = n
        return img

    def writing_boundary(self, lb_field, path="boundary.npy"):
        """Headless replacement of the reference's PNG dump (:486-510)."""
        np.save(path, self.group_map(lb_field))
        return path
