"""``jax.numpy`` stand-in backed by NumPy; see ``jax/__init__.py``.

Arrays are :class:`Array`, an ``ndarray`` subclass that adds JAX's functional
``x.at[idx].set(v)`` update and makes augmented assignment rebind instead of
mutating (JAX arrays are immutable).
"""

from __future__ import annotations

import numpy as _np


class _AtIndexer:
    def __init__(self, arr, idx):
        self.arr = arr
        self.idx = idx

    def set(self, value, **kwargs):
        out = _np.array(self.arr, copy=True).view(Array)
        out[self.idx] = value
        return out

    def add(self, value, **kwargs):
        out = _np.array(self.arr, copy=True).view(Array)
        out[self.idx] += value
        return out

    def get(self, **kwargs):
        return self.arr[self.idx]


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIndexer(self.arr, idx)


class Array(_np.ndarray):
    @property
    def at(self):
        return _At(self)

    def __iadd__(self, other):
        return _np.add(self, other)

    def __isub__(self, other):
        return _np.subtract(self, other)

    def __imul__(self, other):
        return _np.multiply(self, other)

    def __itruediv__(self, other):
        return _np.true_divide(self, other)


def _wrap(x):
    if isinstance(x, _np.ndarray) and not isinstance(x, Array):
        return x.view(Array)
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, list):
        return [_wrap(v) for v in x]
    return x


def _wrapped(fn):
    def inner(*args, **kwargs):
        return _wrap(fn(*args, **kwargs))

    inner.__name__ = getattr(fn, "__name__", "fn")
    return inner


def array(obj, dtype=None, **kwargs):
    return _np.array(obj, dtype=dtype).view(Array)


def asarray(obj, dtype=None, **kwargs):
    return _np.asarray(obj, dtype=dtype).view(Array)


def convolve(a, v, mode="full", **kwargs):
    return _np.convolve(_np.asarray(a), _np.asarray(v), mode=mode).view(Array)


linalg = _np.linalg
s_ = _np.s_
index_exp = _np.index_exp
inf = _np.inf
pi = _np.pi
e = _np.e
newaxis = None
dtype = _np.dtype
finfo = _np.finfo
iinfo = _np.iinfo
float32 = _np.float32
float64 = _np.float64
int32 = _np.int32
int64 = _np.int64
complex64 = _np.complex64
complex128 = _np.complex128
bool_ = _np.bool_
ndarray = Array


def __getattr__(name):
    obj = getattr(_np, name)
    if callable(obj) and not isinstance(obj, type):
        return _wrapped(obj)
    return obj
