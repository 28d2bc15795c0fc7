"""Flux and slope limiters of the MUSCL reconstructions (mirrors
``src/pyshocks/limiters.py``). The limiter arithmetic runs inside the flux
kernels; these frozen dataclasses carry the choice and its parameter."""

from __future__ import annotations

from dataclasses import dataclass, fields
from typing import Any

from pyshocks_gb300 import _lib as L


@dataclass(frozen=True)
class Limiter:
    """``src/pyshocks/limiters.py:43-73``."""

    code = L.SHK_LIM_NONE

    @property
    def is_symmetric(self) -> bool:
        return False

    @property
    def param(self) -> float:
        """The parameter passed to the kernels (theta / variant)."""
        return 1.0


@dataclass(frozen=True)
class UnlimitedLimiter(Limiter):
    """``src/pyshocks/limiters.py:132-155``."""


@dataclass(frozen=True)
class MINMODLimiter(Limiter):
    """``max(0, min(theta, theta r, (1 + r)/2))``, theta in [1, 2]
    (``src/pyshocks/limiters.py:166-209``)."""

    theta: float = 1.0
    code = L.SHK_LIM_MINMOD

    def __post_init__(self) -> None:
        if self.theta < 1.0 or self.theta > 2.0:
            raise ValueError(f"'theta' must be in [1, 2]: {self.theta!r}.")

    @property
    def is_symmetric(self) -> bool:
        return True

    @property
    def param(self) -> float:
        return float(self.theta)


@dataclass(frozen=True)
class MonotonizedCentralLimiter(Limiter):
    """``src/pyshocks/limiters.py:215-245``."""

    code = L.SHK_LIM_MC

    @property
    def is_symmetric(self) -> bool:
        return True


@dataclass(frozen=True)
class SUPERBEELimiter(Limiter):
    """``src/pyshocks/limiters.py:251-278``."""

    code = L.SHK_LIM_SUPERBEE

    @property
    def is_symmetric(self) -> bool:
        return True


@dataclass(frozen=True)
class VanAlbadaLimiter(Limiter):
    """``src/pyshocks/limiters.py:284-339``; variant 2 is not symmetric."""

    variant: int = 1
    code = L.SHK_LIM_VANALBADA

    def __post_init__(self) -> None:
        if self.variant not in {1, 2}:
            raise ValueError(f"Variants 1 and 2 are supported: {self.variant}")

    @property
    def is_symmetric(self) -> bool:
        return self.variant == 1

    @property
    def param(self) -> float:
        return float(self.variant)


@dataclass(frozen=True)
class VanLeerLimiter(Limiter):
    """``src/pyshocks/limiters.py:345-375``."""

    code = L.SHK_LIM_VANLEER

    @property
    def is_symmetric(self) -> bool:
        return True


@dataclass(frozen=True)
class KorenLimiter(Limiter):
    """``src/pyshocks/limiters.py:381-388`` (flux limiter only)."""

    code = L.SHK_LIM_KOREN


_LIMITERS: dict[str, type[Limiter]] = {
    "default": MINMODLimiter,
    "none": UnlimitedLimiter,
    "minmod": MINMODLimiter,
    "mc": MonotonizedCentralLimiter,
    "superbee": SUPERBEELimiter,
    "vanalbada": VanAlbadaLimiter,
    "vanleer": VanLeerLimiter,
    "koren": KorenLimiter,
}


def limiter_ids() -> tuple[str, ...]:
    return tuple(_LIMITERS)


def make_limiter_from_name(name: str, **kwargs: Any) -> Limiter:
    """``src/pyshocks/limiters.py:417-432``: unknown keyword arguments are ignored."""
    cls = _LIMITERS.get(name)
    if cls is None:
        raise ValueError(f"Limiter {name!r} not found. Try one of {', '.join(limiter_ids())}.")
    return cls(**{f.name: kwargs[f.name] for f in fields(cls) if f.name in kwargs})
