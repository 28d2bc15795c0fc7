"""Reconstructions on the GB300 path (mirrors ``src/pyshocks/reconstruction.py``).

The reconstruction objects are the reference's frozen dataclasses; the
arithmetic runs inside the flux kernels of ``libshocks.so`` (there is no
standalone reconstruction kernel: ul/ur never leave shared memory).
"""

from __future__ import annotations

from dataclasses import dataclass, fields
from typing import Any

from pyshocks_gb300 import _lib as L


@dataclass(frozen=True)
class Reconstruction:
    """``src/pyshocks/reconstruction.py:48-76``."""

    @property
    def name(self) -> str:
        return type(self).__name__.lower()

    @property
    def order(self) -> int:
        raise NotImplementedError(type(self).__name__)

    @property
    def stencil_width(self) -> int:
        raise NotImplementedError(type(self).__name__)


@dataclass(frozen=True)
class ConstantReconstruction(Reconstruction):
    """First-order constant reconstruction, ``ul = ur = u``
    (``src/pyshocks/reconstruction.py:128-163``)."""

    @property
    def name(self) -> str:
        return "constant"

    @property
    def order(self) -> int:
        return 1

    @property
    def stencil_width(self) -> int:
        return 1

    code = L.SHK_REC_CONSTANT


@dataclass(frozen=True)
class WENOJS(Reconstruction):
    """``src/pyshocks/reconstruction.py:305-317``."""

    eps: float

    @property
    def stencil_width(self) -> int:
        return self.order


@dataclass(frozen=True)
class WENOJS32(WENOJS):
    """Third-order WENO-JS, second order in non-smooth regions
    (``src/pyshocks/reconstruction.py:320-333``)."""

    eps: float = 1.0e-6

    @property
    def order(self) -> int:
        return 2

    code = L.SHK_REC_WENOJS32


@dataclass(frozen=True)
class WENOJS53(WENOJS):
    """Fifth-order WENO-JS (``src/pyshocks/reconstruction.py:335-348``)."""

    eps: float = 1.0e-12

    @property
    def order(self) -> int:
        return 3

    code = L.SHK_REC_WENOJS53


@dataclass(frozen=True)
class ESWENO32(Reconstruction):
    """ES-WENO weights of [Yamaleev2009] (``src/pyshocks/reconstruction.py:386-411``)."""

    eps: float = 1.0e-6
    delta: float = 1.0e-6

    @property
    def order(self) -> int:
        return 2

    @property
    def stencil_width(self) -> int:
        return 2

    code = L.SHK_REC_ESWENO32


@dataclass(frozen=True)
class MUSCL(Reconstruction):
    """Second-order MUSCL with a flux limiter on the slope ratio
    (``src/pyshocks/reconstruction.py:172-245``)."""

    lm: Any = None
    atol: float = 1.0e-12

    def __post_init__(self) -> None:
        if self.lm is None:
            from pyshocks_gb300.limiters import MINMODLimiter

            object.__setattr__(self, "lm", MINMODLimiter(theta=1.0))

    @property
    def name(self) -> str:
        return f"{type(self).__name__}_{type(self.lm).__name__[:-7]}".lower()

    @property
    def order(self) -> int:
        return 2

    @property
    def stencil_width(self) -> int:
        return 2

    code = L.SHK_REC_MUSCL


@dataclass(frozen=True)
class MUSCLS(MUSCL):
    """Second-order MUSCL with a slope limiter
    (``src/pyshocks/reconstruction.py:251-290``)."""

    code = L.SHK_REC_MUSCLS

    def __post_init__(self) -> None:
        super().__post_init__()
        if type(self.lm).__name__ == "KorenLimiter":
            raise NotImplementedError("the Koren limiter has no slope form")


_RECONSTRUCTION: dict[str, type[Reconstruction]] = {
    "default": ConstantReconstruction,
    "constant": ConstantReconstruction,
    "wenojs32": WENOJS32,
    "wenojs53": WENOJS53,
    "esweno32": ESWENO32,
    "muscl": MUSCL,
    "muscls": MUSCLS,
}


def reconstruction_ids() -> tuple[str, ...]:
    return tuple(_RECONSTRUCTION)


def make_reconstruction_from_name(name: str, **kwargs: Any) -> Reconstruction:
    """``src/pyshocks/reconstruction.py:547-566``: unknown keyword arguments are
    ignored, as in the reference."""
    cls = _RECONSTRUCTION.get(name)
    if cls is None and name == "ssweno242":
        # the reference's entropy-stable SBP reconstruction: not on this path
        raise NotImplementedError(
            f"Reconstruction {name!r} (summation-by-parts) has no GPU implementation. "
            f"Try one of {', '.join(reconstruction_ids())}.")
    if cls is None:
        raise ValueError(
            f"Reconstruction {name!r} not found. Try one of {', '.join(reconstruction_ids())}."
        )
    return cls(**{f.name: kwargs[f.name] for f in fields(cls) if f.name in kwargs})
