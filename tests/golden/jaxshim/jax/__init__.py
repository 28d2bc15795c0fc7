"""A NumPy-backed stand-in for the few ``jax`` entry points that pyshocks'
forward path uses, so that the reference's own Python source can be imported
and executed in a container without JAX to generate golden vectors.

Test infrastructure only (used by ``tests/golden/make_golden.py``). It is not
JAX: ``jit`` is the identity, arrays are NumPy arrays with a functional
``.at[...].set`` helper, and reductions/convolutions follow NumPy's summation
order rather than XLA's.
"""

from __future__ import annotations

import functools
import types

import numpy as _np

from . import numpy  # noqa: F401
from .numpy import Array  # noqa: F401
from . import scipy  # noqa: F401


class _Config:
    def update(self, name, val=None):
        return None


config = _Config()


def jit(fun=None, **kwargs):
    if fun is None:
        return lambda f: f
    return fun


def device_put(x, *args, **kwargs):
    return numpy.asarray(x)


def device_get(x):
    return _np.asarray(x)


def jacfwd(*args, **kwargs):
    raise NotImplementedError("jacfwd is not available in the NumPy stand-in")


def vjp(*args, **kwargs):
    raise NotImplementedError("vjp is not available in the NumPy stand-in")


def _fori_loop(lower, upper, body, init):
    val = init
    for i in range(lower, upper):
        val = body(i, val)
    return val


lax = types.SimpleNamespace(fori_loop=_fori_loop)
tree_util = types.SimpleNamespace(
    register_pytree_node=lambda *a, **k: None,
    register_pytree_node_class=lambda cls: cls,
)
Array = numpy.Array
