"""Uniform cell grids, quadrature and norms (mirrors ``src/pyshocks/grid.py``).

Grid arrays are torch tensors on the CUDA device; the layout is the
reference's: ``n`` interior cells plus ``nghosts`` ghost cells on each side.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Callable

import numpy as np
import torch


@dataclass(frozen=True)
class Grid:
    """``src/pyshocks/grid.py:47-117``."""

    a: float
    b: float
    nghosts: int
    x: torch.Tensor
    dx: torch.Tensor
    f: torch.Tensor
    df: torch.Tensor
    dx_min: float
    dx_max: float
    is_periodic: bool

    @property
    def dtype(self) -> torch.dtype:
        return self.x.dtype

    @property
    def n(self) -> int:
        """Number of cells including ghosts (``grid.py:79-81``)."""
        return int(self.x.numel())

    @property
    def ncells(self) -> int:
        """Number of interior cells."""
        return int(self.x.numel()) - 2 * self.nghosts

    @property
    def i_(self) -> slice:
        return slice(self.nghosts, self.x.numel() - self.nghosts)

    @property
    def f_(self) -> slice:
        return slice(self.nghosts, self.f.numel() - self.nghosts)

    @property
    def g_(self) -> tuple[None, slice, slice]:
        n = self.x.numel()
        return (None, slice(n - self.nghosts, n), slice(0, self.nghosts))

    @property
    def gi_(self) -> tuple[None, slice, slice]:
        g = self.nghosts
        n = self.x.numel()
        return (None, slice(n - 2 * g, n - g), slice(g, 2 * g))


@dataclass(frozen=True)
class UniformGrid(Grid):
    pass


def _device(device: Any) -> torch.device:
    return torch.device(device) if device is not None else torch.device("cuda")


def make_uniform_cell_grid(
    a: float,
    b: float,
    n: int,
    *,
    nghosts: int = 1,
    dtype: Any = None,
    device: Any = None,
) -> UniformGrid:
    """``src/pyshocks/grid.py:131-179``; coordinates are generated in float64
    on the host (as the reference's ``jnp.linspace``) and moved to *device*."""
    if b < a:
        raise ValueError(f"Incorrect interval a > b: {a!r} > {b!r}.")
    if n <= 0:
        raise ValueError(f"Number of cells should be > 0: {n!r} <= 0.")
    dtype = dtype or torch.float64
    h = (b - a) / n
    f = np.linspace(a - nghosts * h, b + nghosts * h, n + 2 * nghosts + 1)
    x = (f[1:] + f[:-1]) / 2
    df = np.diff(x)
    dx = np.full_like(x, h)
    dev = _device(device)

    def t(v):
        return torch.as_tensor(v, dtype=dtype, device=dev)

    return UniformGrid(
        a=a, b=b, nghosts=nghosts, x=t(x), dx=t(dx), f=t(f), df=t(df),
        dx_min=h, dx_max=h, is_periodic=False,
    )


# {{{ quadrature


@dataclass(frozen=True)
class Quadrature:
    order: int
    x: np.ndarray
    w: np.ndarray
    dx: np.ndarray

    def __call__(self, fn: Callable, axis: int | None = None) -> np.ndarray:
        return np.sum(fn(self.x) * self.w, axis=axis)


def make_leggauss_quadrature(grid: Grid, order: int) -> Quadrature:
    """Gauss-Legendre nodes per cell (``src/pyshocks/grid.py:393-423``)."""
    if order < 1:
        raise ValueError(f"Invalid order: {order!r}.")
    from numpy.polynomial.legendre import leggauss

    f = grid.f.detach().cpu().double().numpy()
    xi, wi = leggauss(order)
    xi = xi.reshape(-1, 1)
    wi = wi.reshape(-1, 1)
    dx = f[1:] - f[:-1]
    dxm = 0.5 * dx.reshape(1, -1)
    xm = 0.5 * (f[1:] + f[:-1]).reshape(1, -1)
    return Quadrature(order=order, x=xm + dxm * xi, w=dxm * wi, dx=dx)


def cell_average(quad: Quadrature, fn: Callable, *, like: torch.Tensor | None = None):
    """Cell averages ``quad(fn) / dx`` (``src/pyshocks/grid.py:426-435``),
    evaluated on the host; returned on *like*'s device/dtype when given."""
    v = quad(fn, axis=0) / quad.dx
    if like is not None:
        return torch.as_tensor(v, dtype=like.dtype, device=like.device)
    return v


# }}}


# {{{ norms


def norm(grid: Grid, u, *, p: Any = 1, weighted: bool = False):
    """Interior norms (``src/pyshocks/grid.py:444-506``); FP64 accumulation."""
    if not isinstance(u, torch.Tensor) or u.dim() == 0:
        return torch.as_tensor(abs(float(u)), dtype=torch.float64)
    if u.shape[0] == grid.x.shape[0]:
        v = u[grid.i_]
        w = grid.dx[grid.i_] if weighted else None
    elif u.shape[0] == grid.f.shape[0]:
        v = u[grid.f_]
        w = grid.df[grid.f_] if weighted else None
    else:
        raise ValueError(f"Array has unexpected shape: {tuple(u.shape[:1])}")
    v = v.double().abs()
    w = 1.0 if w is None else w.double()
    if p == 1:
        return torch.sum(v * w)
    if p == 2:
        return torch.sqrt(torch.sum(v**2 * w))
    if p in {np.inf, "inf"}:
        return torch.max(v)
    if p in {-np.inf, "-inf"}:
        return torch.min(v)
    if p == "tvd":
        return torch.sum(torch.abs(torch.diff(v)))
    if isinstance(p, (int, float)) and p > 0:
        return torch.sum(v**p * w) ** (1.0 / p)
    raise ValueError(f"Unrecognized norm order 'p': {p!r}.")


def rnorm(grid: Grid, u, v, *, p: Any = 1, weighted: bool = False, atol: float = 1.0e-14):
    """``src/pyshocks/grid.py:509-531``."""
    vnorm = norm(grid, v, p=p, weighted=weighted)
    if vnorm < atol:
        vnorm = torch.ones_like(vnorm)
    return norm(grid, u - v, p=p, weighted=weighted) / vnorm


# }}}
