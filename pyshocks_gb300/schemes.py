"""Scheme and boundary generics: the plug-in API of ``src/pyshocks/schemes.py``.

The same ``functools.singledispatch`` generics as the reference
(``bind``, ``apply_operator``, ``predict_timestep``, ``flux``,
``numerical_flux``, ``apply_boundary``, ``evaluate_boundary``). The schemes of
the hot path (``pyshocks_gb300.burgers``) register CUDA implementations; user
schemes can register their own exactly as with the reference.
"""

from __future__ import annotations

import enum
from abc import ABC, abstractmethod
from dataclasses import dataclass
from functools import singledispatch
from typing import TYPE_CHECKING, Any, TypeVar

if TYPE_CHECKING:
    import torch

    from pyshocks_gb300.grid import Grid
    from pyshocks_gb300.reconstruction import Reconstruction


@dataclass(frozen=True)
class SchemeBase:
    """``src/pyshocks/schemes.py:78-118``."""

    rec: Reconstruction

    @property
    def name(self) -> str:
        return f"{type(self).__name__}_{self.rec.name}".lower()

    @property
    def order(self) -> int:
        return self.rec.order

    @property
    def stencil_width(self) -> int:
        return self.rec.stencil_width


SchemeT = TypeVar("SchemeT", bound=SchemeBase)


@singledispatch
def bind(scheme: SchemeBase, grid: Grid, bc: Boundary) -> SchemeBase:
    """``src/pyshocks/schemes.py:124-139``."""
    if isinstance(scheme, SchemeBase):
        return scheme
    raise NotImplementedError(type(scheme).__name__)


@singledispatch
def apply_operator(scheme: SchemeBase, grid: Grid, bc: Boundary, t: Any, u: torch.Tensor):
    """``src/pyshocks/schemes.py:142-166``."""
    raise NotImplementedError(type(scheme).__name__)


@singledispatch
def predict_timestep(scheme: SchemeBase, grid: Grid, bc: Boundary, t: Any, u: torch.Tensor):
    """``src/pyshocks/schemes.py:169-190``."""
    raise NotImplementedError(type(scheme).__name__)


@dataclass(frozen=True)
class FiniteVolumeSchemeBase(SchemeBase):
    """``src/pyshocks/schemes.py:193-199``."""


@dataclass(frozen=True)
class ConservationLawScheme(FiniteVolumeSchemeBase):
    """``src/pyshocks/schemes.py:287-302``."""


@singledispatch
def flux(scheme: SchemeBase, t: Any, x: Any, u: torch.Tensor):
    """``src/pyshocks/schemes.py:305-318``."""
    raise NotImplementedError(type(scheme).__name__)


@singledispatch
def numerical_flux(scheme: SchemeBase, grid: Grid, bc: Boundary, t: Any, u: torch.Tensor):
    """``src/pyshocks/schemes.py:321-336``."""
    raise NotImplementedError(type(scheme).__name__)


@apply_operator.register(ConservationLawScheme)
def _apply_operator_conservation_law(scheme, grid, bc, t, u):
    """Generic conservation-law operator for user-registered fluxes
    (``src/pyshocks/schemes.py:339-346``). The schemes of the hot path register
    a fused CUDA kernel instead."""
    u = apply_boundary(bc, grid, t, u)
    f = numerical_flux(scheme, grid, bc, t, u)
    return -(f[1:] - f[:-1]) / grid.dx


@enum.unique
class BoundaryType(enum.Enum):
    """``src/pyshocks/schemes.py:393-416``."""

    Periodic = enum.auto()
    Dirichlet = enum.auto()
    Neumann = enum.auto()
    HomogeneousNeumann = enum.auto()


@dataclass(frozen=True)
class Boundary(ABC):
    """``src/pyshocks/schemes.py:419-428``."""

    @property
    @abstractmethod
    def boundary_type(self) -> BoundaryType:
        """The broad class of the boundary condition."""


@singledispatch
def apply_boundary(bc: Boundary, grid: Grid, t: Any, u: torch.Tensor):
    """``src/pyshocks/schemes.py:431-442``."""
    raise NotImplementedError(type(bc).__name__)


@singledispatch
def evaluate_boundary(bc: Boundary, grid: Grid, t: Any, u: torch.Tensor):
    """``src/pyshocks/schemes.py:445-456``."""
    raise NotImplementedError(type(bc).__name__)
