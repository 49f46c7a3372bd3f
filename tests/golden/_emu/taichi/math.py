"""taichi.math subset for the serial Taichi stand-in (fixture generation only)."""
import math as _m

import numpy as np

pi = _m.pi
vec2 = "vec2"
vec3 = "vec3"


def dot(a, b):
    """Sequential sum of products, as a Taichi dot of small vectors."""
    acc = a[0] * b[0]
    for k in range(1, len(a)):
        acc = acc + a[k] * b[k]
    return acc


def sqrt(x):
    if isinstance(x, float):
        return _m.sqrt(x)
    return np.sqrt(x)


def exp(x):
    if isinstance(x, float):
        return _m.exp(x)
    return np.exp(x)


def log(x):
    if isinstance(x, float):
        return _m.log(x)
    return np.log(x)


def cos(x):
    return np.cos(x)


def sin(x):
    return np.sin(x)


def floor(x):
    return np.floor(x)


def ceil(x):
    return np.ceil(x)
