"""Boundary conditions of the GB300 path (mirrors ``src/pyshocks/scalar.py``).

Periodic boundaries are applied by the kernels themselves (circular indexing of
the interior cells); :func:`apply_boundary` on a :class:`PeriodicBoundary` is
still provided for user code and generic schemes.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Callable

import torch

from pyshocks_gb300.schemes import Boundary, BoundaryType, apply_boundary, evaluate_boundary


@dataclass(frozen=True)
class PeriodicBoundary(Boundary):
    """``src/pyshocks/scalar.py:520-526``."""

    @property
    def boundary_type(self) -> BoundaryType:
        return BoundaryType.Periodic


@apply_boundary.register(PeriodicBoundary)
def _apply_boundary_scalar_periodic(bc, grid, t, u: torch.Tensor) -> torch.Tensor:
    """``src/pyshocks/scalar.py:529-540``: right ghosts, then left ghosts."""
    assert u.shape[0] == grid.x.shape[0]
    u = u.clone()
    for side in (+1, -1):
        u[grid.g_[side]] = u[grid.gi_[-side]]
    return u


@evaluate_boundary.register(PeriodicBoundary)
def _evaluate_boundary_scalar_periodic(bc, grid, t, u):
    return torch.zeros_like(u)


# {{{ one- and two-sided boundaries (src/pyshocks/scalar.py:345-511)


@dataclass(frozen=True)
class OneSidedBoundary(Boundary):
    """``src/pyshocks/scalar.py:345-356``: *side* is -1 (left) or +1 (right)."""

    side: int

    def __post_init__(self) -> None:
        if self.side not in (-1, +1):
            raise ValueError(f"unknown side: {self.side}")


@dataclass(frozen=True)
class TwoSidedBoundary(Boundary):
    """``src/pyshocks/scalar.py:359-382``: the left boundary, then the right."""

    left: OneSidedBoundary
    right: OneSidedBoundary

    def __post_init__(self) -> None:
        if self.left.side != -1 or self.right.side != +1:
            raise ValueError("left/right boundaries have the wrong sides")

    @property
    def boundary_type(self) -> BoundaryType:
        if self.left.boundary_type == self.right.boundary_type:
            return self.left.boundary_type
        raise ValueError("the two sides have different boundary types")


@apply_boundary.register(TwoSidedBoundary)
def _apply_boundary_two_sided(bc, grid, t, u):
    u = apply_boundary(bc.left, grid, t, u)
    return apply_boundary(bc.right, grid, t, u)


@dataclass(frozen=True)
class DirichletBoundary(OneSidedBoundary):
    """``src/pyshocks/scalar.py:397-413``: ``u(t, a) = g(t, x)`` in the ghost
    cells; ``g`` takes the time and a tensor of ghost-cell centres."""

    g: Callable = None

    @property
    def boundary_type(self) -> BoundaryType:
        return BoundaryType.Dirichlet


@apply_boundary.register(DirichletBoundary)
def _apply_boundary_dirichlet(bc, grid, t, u):
    """``src/pyshocks/scalar.py:416-424``."""
    u = u.clone()
    ito = grid.g_[bc.side]
    u[ito] = torch.as_tensor(bc.g(t, grid.x[ito]), dtype=u.dtype, device=u.device)
    return u


def make_dirichlet_boundary(ga: Callable, gb: Callable | None = None) -> TwoSidedBoundary:
    """``src/pyshocks/scalar.py:427-434``."""
    return TwoSidedBoundary(left=DirichletBoundary(side=-1, g=ga),
                            right=DirichletBoundary(side=+1, g=ga if gb is None else gb))


@dataclass(frozen=True)
class NeumannBoundary(OneSidedBoundary):
    """``src/pyshocks/scalar.py:443-464``: ``+-du/dx(t, a) = g(t)`` with the
    ghost cells mirrored about the boundary face."""

    g: Callable = None

    @property
    def boundary_type(self) -> BoundaryType:
        return BoundaryType.Neumann


@apply_boundary.register(NeumannBoundary)
def _apply_boundary_neumann(bc, grid, t, u):
    """``src/pyshocks/scalar.py:467-495``."""
    u = u.clone()
    g = grid.nghosts
    n = u.shape[0]
    ifrom = torch.arange(*grid.gi_[bc.side].indices(n), device=u.device)
    if bc.side == -1:
        ito = torch.arange(g - 1, -1, -1, device=u.device)
    else:
        ito = torch.arange(n - 1, n - g - 1, -1, device=u.device)
    gn = float(bc.g(t))
    u[ito] = u[ifrom] + bc.side * (grid.x[ifrom] - grid.x[ito]) * gn
    return u


def make_neumann_boundary(ga: Callable, gb: Callable | None = None) -> TwoSidedBoundary:
    """``src/pyshocks/scalar.py:498-505``."""
    return TwoSidedBoundary(left=NeumannBoundary(side=-1, g=ga),
                            right=NeumannBoundary(side=+1, g=ga if gb is None else gb))


# }}}
