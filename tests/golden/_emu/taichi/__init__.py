"""Minimal serial stand-in for the Taichi runtime, used ONLY to execute the
reference's own Python source (taichi_lbm/*.py) in a container where Taichi
cannot be installed, so that golden fixtures come from the reference's code.

Test infrastructure, not product code.  It implements just the subset of the
Taichi language that taichi_lbm/ and the fixture drivers use:

* ``ti.field`` / ``ti.Vector.field`` / ``ti.Matrix.field`` backed by numpy,
  with ``offset=`` support and out-of-range indices raising ``IndexError``
  (Taichi itself reads undefined memory there; a fixture must never do so).
* ``@ti.kernel`` / ``@ti.func`` run the Python body serially.  Serial order is
  one legal schedule of Taichi's parallel outer loop; every reference kernel
  used by the fixtures is order-independent (no node of a group reads a value
  another node of the same group writes in the same kernel).
* Arithmetic follows Taichi's typing: ``float`` is the default float type
  (f32 unless ``ti.init(default_fp=ti.f64)``), ``int`` is i32, integer
  constants are weak.  ``x ** <int literal>`` is rewritten to repeated
  multiplication (what Taichi emits for integer exponents) and
  ``ti.atomic_add(a[i], v)`` to a read-modify-write, both by an AST pass.
* No fast-math: every operation is a separately rounded IEEE op in the
  declared precision (numpy semantics).  Real Taichi compiles with fast-math
  (contractions allowed), so the real reference may differ in the last bits.
"""
import ast
import inspect
import math as _pymath
import textwrap

import numpy as np

from . import math  # noqa: F401  (taichi.math)

f32 = np.float32
f64 = np.float64
i32 = np.int32
i64 = np.int64
u8 = np.uint8
gpu = "gpu"
cpu = "cpu"
cuda = "cuda"

_cfg = {"fp": np.float32}


def init(arch=None, default_fp=None, **kwargs):
    """Select the default float type; the arch is ignored (always serial)."""
    if default_fp is not None:
        _cfg["fp"] = np.dtype(default_fp).type
    else:
        _cfg["fp"] = np.float32


def default_fp():
    return _cfg["fp"]


def _dtype(d):
    if d is float:
        return _cfg["fp"]
    if d is int:
        return np.int32
    return np.dtype(d).type


class Vec(np.ndarray):
    """numpy array with Taichi vector conveniences (.x/.y, int elements as
    Python ints so integer constants stay weakly typed, matmul in the float
    type of the operands, sequential reduction order)."""

    def __getitem__(self, key):
        r = super().__getitem__(key)
        if np.ndim(r) == 0 and np.issubdtype(self.dtype, np.integer):
            return int(r)
        return r

    def __iter__(self):
        for k in range(self.shape[0]):
            yield self[k]

    def _get(self, k):
        return self[k]

    def _set(self, k, v):
        self[k] = v

    x = property(lambda s: s._get(0), lambda s, v: s._set(0, v))
    y = property(lambda s: s._get(1), lambda s, v: s._set(1, v))
    z = property(lambda s: s._get(2), lambda s, v: s._set(2, v))

    def __matmul__(self, other):
        a = np.asarray(self)
        b = np.asarray(other)
        if np.issubdtype(a.dtype, np.floating) or np.issubdtype(b.dtype, np.floating):
            dt = a.dtype if np.issubdtype(a.dtype, np.floating) else b.dtype
        else:
            dt = np.int32
        a = a.astype(dt)
        b = b.astype(dt)
        if a.ndim == 2 and b.ndim == 1:
            out = np.zeros(a.shape[0], dt)
            for r in range(a.shape[0]):
                acc = dt.type(0) if hasattr(dt, "type") else dt(0)
                acc = a[r, 0] * b[0]
                for c in range(1, a.shape[1]):
                    acc = acc + a[r, c] * b[c]
                out[r] = acc
            return out.view(Vec)
        raise NotImplementedError("only matrix @ vector is emulated")


def _vec(values, dtype=None):
    if dtype is None:
        flat = np.asarray(values, dtype=object).ravel()
        is_int = all(isinstance(v, (int, np.integer)) and not isinstance(v, bool) for v in flat)
        dtype = np.int32 if is_int else _cfg["fp"]
    return np.array(values, dtype=dtype).view(Vec)


class _Template:
    pass


def template():
    return _Template()


def static(x, *args):
    return x


class Field:
    """Dense field over an index box, optionally with a vector/matrix element."""

    def __init__(self, dtype, shape, elem=(), offset=None):
        if isinstance(shape, (int, np.integer)):
            shape = (int(shape),)
        self.shape = tuple(int(s) for s in shape)
        self.offset = tuple(offset) if offset is not None else (0,) * len(self.shape)
        self.dtype = _dtype(dtype)
        self.elem = tuple(elem)
        self.arr = np.zeros(self.shape + self.elem, self.dtype)

    def _idx(self, key):
        if key is None:
            return ()
        if not isinstance(key, tuple):
            key = (key,)
        idx = []
        for k, o, n in zip(key, self.offset, self.shape):
            v = int(k) - o
            if v < 0 or v >= n:
                raise IndexError(f"field index {tuple(key)} outside [{self.offset}, +{self.shape})")
            idx.append(v)
        return tuple(idx)

    def __getitem__(self, key):
        idx = self._idx(key)
        if self.elem:
            return self.arr[idx].view(Vec)
        r = self.arr[idx]
        if np.issubdtype(self.dtype, np.integer):
            return int(r)
        return self.dtype(r)

    def __setitem__(self, key, val):
        self.arr[self._idx(key)] = val

    def fill(self, v):
        self.arr[...] = v

    def to_numpy(self):
        return self.arr.copy()

    def from_numpy(self, a):
        self.arr[...] = a

    def __iter__(self):
        for ix in np.ndindex(*self.shape):
            yield tuple(int(a) + o for a, o in zip(ix, self.offset))


def field(dtype, shape=(), offset=None, **kwargs):
    return Field(dtype, shape, (), offset)


class Vector:
    def __new__(cls, values, dt=None):
        return _vec(values, None if dt is None else _dtype(dt))

    @staticmethod
    def field(n, dtype, shape=(), offset=None, **kwargs):
        return Field(dtype, shape, (n,), offset)


class Matrix:
    def __new__(cls, values, dt=None):
        return _vec(values, None if dt is None else _dtype(dt))

    @staticmethod
    def field(n, m, dtype, shape=(), offset=None, **kwargs):
        return Field(dtype, shape, (n, m), offset)


class types:
    @staticmethod
    def vector(n, dtype):
        def ctor(*vals):
            if len(vals) == 1 and np.ndim(vals[0]) == 1:
                vals = tuple(vals[0])
            return _vec(list(vals), _dtype(dtype))
        return ctor

    @staticmethod
    def matrix(n, m, dtype):
        def ctor(*rows):
            return _vec([list(r) for r in rows], _dtype(dtype))
        return ctor


def data_oriented(cls):
    return cls


class StructField:
    """A field of ti.dataclass structs: one Field per member."""

    def __init__(self, members, shape, offset=None):
        object.__setattr__(self, "_members",
                           {name: Field(dt, shape, elem, offset) for name, (elem, dt) in members.items()})

    def __getitem__(self, key):
        return _StructRef(self, key)

    def __getattr__(self, name):
        try:
            return object.__getattribute__(self, "_members")[name]
        except KeyError:
            raise AttributeError(name) from None

    def __iter__(self):
        return iter(next(iter(self._members.values())))


class _StructRef:
    """One struct of a StructField: members read as views (so .x/.y writes land
    in the field) and assignments write through."""

    __slots__ = ("_sf", "_key")

    def __init__(self, sf, key):
        object.__setattr__(self, "_sf", sf)
        object.__setattr__(self, "_key", key)

    def __getattr__(self, name):
        f = self._sf._members[name]
        idx = f._idx(self._key)
        if f.elem:
            return f.arr[idx].view(Vec)
        r = f.arr[idx]
        return int(r) if np.issubdtype(f.dtype, np.integer) else f.dtype(r)

    def __setattr__(self, name, value):
        f = self._sf._members[name]
        f.arr[f._idx(self._key)] = value


def dataclass(cls):
    """Struct types: Cls.field(shape=...) gives a StructField whose members
    follow the annotations (ti.math.vec2/vec3 vectors, int, float)."""
    ann = dict(getattr(cls, "__annotations__", {}))

    def field(shape=(), offset=None, **kwargs):
        members = {}
        for name, a in ann.items():
            if a in ("vec2", "vec3"):
                members[name] = ((int(a[-1]),), float)
            elif a is int:
                members[name] = ((), int)
            else:
                members[name] = ((), float)
        return StructField(members, shape, offset)

    cls.field = staticmethod(field)
    return cls


def ndrange(*ranges):
    import itertools
    return itertools.product(*[range(*r) if isinstance(r, tuple) else range(r) for r in ranges])


def cast(x, dtype):
    return int(x) if dtype is int else _dtype(dtype)(x)


def round(x):  # noqa: A001  (taichi's name)
    return np.round(x)


def abs(x):  # noqa: A001  (taichi's name)
    return np.abs(x)


def _ti_ipow(a, n):
    """Integer power by repeated multiplication (x*x, (x*x)*x, ...)."""
    if n == 0:
        return type(a)(1) if not isinstance(a, (int, float)) else 1
    r = a
    for _ in range(n - 1):
        r = r * a
    return r


def _ti_atomic_add(container, key, value):
    old = container[key]
    container[key] = old + value
    return old


def atomic_add(x, v):  # only reached when the first argument is not a subscript
    raise NotImplementedError("ti.atomic_add emulation needs a subscript target")


class _Rewrite(ast.NodeTransformer):
    def visit_Call(self, node):
        self.generic_visit(node)
        f = node.func
        if (isinstance(f, ast.Attribute) and f.attr == "atomic_add"
                and node.args and isinstance(node.args[0], ast.Subscript)):
            sub = node.args[0]
            return ast.copy_location(
                ast.Call(func=ast.Name("_ti_atomic_add", ast.Load()),
                         args=[sub.value, sub.slice, node.args[1]], keywords=[]), node)
        return node

    def visit_BinOp(self, node):
        self.generic_visit(node)
        if (isinstance(node.op, ast.Pow) and isinstance(node.right, ast.Constant)
                and type(node.right.value) is int):
            return ast.copy_location(
                ast.Call(func=ast.Name("_ti_ipow", ast.Load()),
                         args=[node.left, node.right], keywords=[]), node)
        return node


def _transform(fn):
    try:
        src = textwrap.dedent(inspect.getsource(fn))
    except (OSError, TypeError):
        return fn
    if "atomic_add" not in src and "**" not in src:
        return fn
    tree = ast.parse(src)
    fdef = tree.body[0]
    fdef.decorator_list = []
    tree = ast.fix_missing_locations(_Rewrite().visit(tree))
    g = fn.__globals__
    g.setdefault("_ti_ipow", _ti_ipow)
    g.setdefault("_ti_atomic_add", _ti_atomic_add)
    freevars = fn.__code__.co_freevars
    if freevars:
        outer = ast.FunctionDef(
            name="_ti_outer",
            args=ast.arguments(posonlyargs=[], args=[ast.arg(v) for v in freevars],
                               kwonlyargs=[], kw_defaults=[], defaults=[]),
            body=[fdef, ast.Return(ast.Name(fdef.name, ast.Load()))],
            decorator_list=[])
        mod = ast.fix_missing_locations(ast.Module(body=[outer], type_ignores=[]))
        ns = {}
        exec(compile(mod, inspect.getsourcefile(fn) or "<ti>", "exec"), g, ns)
        cells = [c.cell_contents for c in fn.__closure__]
        return ns["_ti_outer"](*cells)
    ns = {}
    exec(compile(tree, inspect.getsourcefile(fn) or "<ti>", "exec"), g, ns)
    return ns[fdef.name]


def func(fn):
    return _transform(fn)


def kernel(fn):
    body = _transform(fn)
    sig = inspect.signature(fn)

    def run(*args, **kwargs):
        bound = sig.bind(*args, **kwargs)
        for name, p in sig.parameters.items():
            if name not in bound.arguments:
                continue
            ann = p.annotation
            if ann is float:
                bound.arguments[name] = _cfg["fp"](bound.arguments[name])
            elif ann is int:
                bound.arguments[name] = int(bound.arguments[name])
        return body(*bound.args, **bound.kwargs)

    run.__wrapped__ = fn
    return run


def random(dtype=float):
    raise NotImplementedError("fixture drivers seed their own inputs")


def sqrt(x):
    return math.sqrt(x)
