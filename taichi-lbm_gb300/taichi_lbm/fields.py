"""Device fields exposed in taichi-lbm's index order.

The reference's fields are Taichi fields indexed ``[i, j, component]`` with
vector elements innermost (taichi_lbm/lbm.py:22-56).  Here each field is a
PyTorch CUDA tensor in the structure-of-arrays layout of the C ABI
(``[vector][ny][pitch]``, x fastest); :class:`Field` translates reference-order
indexing, ``fill`` and ``to_numpy``/``from_numpy`` onto it.
"""
import numpy as np
import torch


def round_up(v, m):
    return (v + m - 1) // m * m


class Scalar0D:
    """Stand-in for a shape-() Taichi field: ``x[None]`` reads/writes it."""

    def __init__(self, value=0):
        self.value = value

    def __getitem__(self, key):
        return self.value

    def __setitem__(self, key, v):
        self.value = v

    def __int__(self):
        return int(self.value)


class Field:
    """A lattice field.

    kind:
      ``"s"``   scalar per node, reference shape (NX, NY)
      ``"sc"``  scalar per node and component, shape (NX, NY, 1)
      ``"v"``   n-vector per node, shape (NX, NY, n)
      ``"vc"``  n-vector per node and component, shape (NX, NY, 1, n)
    The tensor is ``[ny][pitch]`` (scalars) or ``[n][ny][pitch]`` (vectors);
    ``halo`` = 1 means one extra node on every side (index -1 .. NX).  With
    nc > 1 components the per-component kinds ("sc", "vc") hold a leading
    component axis: ``[nc][ny][pitch]`` / ``[nc][n][ny][pitch]``, shape
    (NX, NY, nc) / (NX, NY, nc, n) in reference order.
    """

    def __init__(self, owner, attr, nx, ny, kind, n=None, halo=0, nc=1):
        self._owner, self._attr = owner, attr
        self.nx, self.ny, self.kind, self.n, self.halo = nx, ny, kind, n, halo
        self.nc = int(nc) if kind in ("sc", "vc") else 1

    @property
    def tensor(self):
        return getattr(self._owner, self._attr)

    @property
    def shape(self):
        nx, ny = self.nx + 2 * self.halo, self.ny + 2 * self.halo
        return {"s": (nx, ny), "sc": (nx, ny, self.nc), "v": (nx, ny, self.n),
                "vc": (nx, ny, self.nc, self.n)}[self.kind]

    def _view(self):
        """Tensor view in reference order (device)."""
        t = self.tensor
        w = self.nx + 2 * self.halo
        if self.nc > 1:
            if self.kind == "sc":  # [nc][ny][pitch] -> (nx, ny, nc)
                return t[:, :, :w].permute(2, 1, 0)
            return t[:, :, :, :w].permute(3, 2, 0, 1)  # [nc][n][ny][pitch] -> (nx, ny, nc, n)
        if self.kind in ("s", "sc"):
            v = t[:, :w].transpose(0, 1)
            return v.unsqueeze(-1) if self.kind == "sc" else v
        v = t[:, :, :w].permute(2, 1, 0)
        return v.unsqueeze(2) if self.kind == "vc" else v

    def to_numpy(self):
        return self._view().contiguous().cpu().numpy()

    def to_torch(self):
        return self._view().contiguous()

    def from_numpy(self, a):
        a = torch.as_tensor(np.asarray(a, dtype=np.float32), device=self.tensor.device)
        self._view().copy_(a.reshape(self.shape))

    def from_torch(self, t, non_blocking=True):
        """Copy a tensor in reference shape (host pinned or device) in."""
        self._view().copy_(t.reshape(self.shape), non_blocking=non_blocking)

    def fill(self, v):
        if self.kind in ("s", "sc"):
            self.tensor.fill_(float(v))
        else:
            vals = np.broadcast_to(np.asarray(v, dtype=np.float32), (self.n,))
            for c in range(self.n):
                if self.nc > 1:
                    self.tensor[:, c].fill_(float(vals[c]))
                else:
                    self.tensor[c].fill_(float(vals[c]))

    def _key(self, key):
        if not isinstance(key, tuple):
            key = (key,)
        if self.nc > 1:
            return None  # indexed through the reference-order copy
        if all(isinstance(k, (int, np.integer)) for k in key):
            i, j = int(key[0]) + self.halo, int(key[1]) + self.halo
            rest = key[2:]
            if self.kind in ("sc", "vc") and rest:
                rest = rest[1:]  # single component
            return i, j, rest
        return None

    def __getitem__(self, key):
        k = self._key(key)
        if k is None:
            return self.to_numpy()[key]
        i, j, rest = k
        t = self.tensor
        if self.kind in ("s", "sc"):
            return float(t[j, i].item())
        vec = t[:, j, i].cpu().numpy()
        return vec[rest] if rest else vec

    def __setitem__(self, key, value):
        k = self._key(key)
        if k is None:
            a = self.to_numpy()
            a[key] = value
            self.from_numpy(a)
            return
        i, j, rest = k
        t = self.tensor
        if self.kind in ("s", "sc"):
            t[j, i] = float(value)
        elif rest:
            t[rest[0], j, i] = float(value)
        else:
            t[:, j, i] = torch.as_tensor(np.asarray(value, np.float32), device=t.device)

    def __array__(self, dtype=None, copy=None):
        a = self.to_numpy()
        return a.astype(dtype) if dtype is not None else a


class MaskField:
    """LBField.mask: host-authoritative int32 (NX, NY), 1 fluid / -1 solid.

    Kept on the host because boundary classification (a setup step) evaluates
    user geometry predicates against it; uploaded when the device needs it.
    Indexing accepts integers or numpy index arrays (vectorised predicates).
    """

    def __init__(self, nx, ny):
        self.arr = np.ones((nx, ny), np.int32)
        self.version = 0

    shape = property(lambda self: self.arr.shape)

    def __getitem__(self, key):
        return self.arr[key]

    def __setitem__(self, key, v):
        self.arr[key] = v
        self.version += 1

    def fill(self, v):
        self.arr[...] = v
        self.version += 1

    def to_numpy(self):
        return self.arr.copy()

    def from_numpy(self, a):
        self.arr[...] = a
        self.version += 1

    def __array__(self, dtype=None, copy=None):
        return self.arr if dtype is None else self.arr.astype(dtype)


def alloc(shape, device, dtype=torch.float32):
    return torch.zeros(shape, dtype=dtype, device=device)
