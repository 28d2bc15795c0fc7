"""Boundary conditions of the GB300 path (mirrors ``src/pyshocks/scalar.py``).

Periodic boundaries are applied by the kernels themselves (circular indexing of
the interior cells); :func:`apply_boundary` on a :class:`PeriodicBoundary` is
still provided for user code and generic schemes.
"""

from __future__ import annotations

from dataclasses import dataclass

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
