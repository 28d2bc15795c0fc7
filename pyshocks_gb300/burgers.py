"""Schemes on the GB300 path (mirrors ``src/pyshocks/burgers/schemes.py`` plus
the flux plug-ins used by the batched workloads).

Each scheme class is the reference's frozen dataclass; ``apply_operator``,
``predict_timestep`` and ``numerical_flux`` are registered with CUDA
implementations from ``libshocks.so``. The physical flux is selected by the
class: Burgers ``u^2/2`` (``burgers/schemes.py:37-39``), linear advection
``c u`` and LWR traffic ``u (1 - u)`` (the plug-in pattern of
``examples/traffic-flow-model.py:14-39``).
"""

from __future__ import annotations

import ctypes

from dataclasses import dataclass, fields, replace
from typing import Any, ClassVar

import torch

from pyshocks_gb300 import _lib as L
from pyshocks_gb300 import reconstruction as rec_mod
from pyshocks_gb300.grid import Grid
from pyshocks_gb300.scalar import (
    DirichletBoundary,
    NeumannBoundary,
    PeriodicBoundary,
    TwoSidedBoundary,
)
from pyshocks_gb300.schemes import (
    Boundary,
    ConservationLawScheme,
    SchemeBase,
    apply_operator,
    bind,
    flux,
    predict_timestep,
)


@dataclass(frozen=True)
class GpuConservationLawScheme(ConservationLawScheme):
    """Base of the schemes whose operator runs in ``libshocks.so``."""

    equation_code: ClassVar[int] = L.SHK_EQ_BURGERS
    flux_code: ClassVar[int] = L.SHK_FLUX_RUSANOV

    @property
    def speed(self) -> float:
        return 1.0

    def nu_for(self, dx: float) -> float:
        """Artificial viscosity factor of the Rusanov flux (1 by default)."""
        return 1.0

    def cfl_constant(self, dx: float) -> float:
        """``0.5 dx^(2 - alpha)`` of the CFL estimate."""
        return 0.5 * dx

    def c_scheme(self, dx: float = 1.0) -> L.ShkScheme:
        rec = self.rec
        s = L.ShkScheme()
        s.flux = self.flux_code
        s.rec = getattr(rec, "code", -1)
        s.equation = self.equation_code
        s.eps = float(getattr(rec, "eps", 1.0e-6))
        s.delta = float(getattr(rec, "delta", 0.0))
        if isinstance(rec, rec_mod.MUSCL):
            # the limiter, its parameter and the slope-ratio cut
            s.limiter = int(rec.lm.code)
            s.delta = float(rec.lm.param)
            s.eps = float(rec.atol)
        s.nu = float(self.nu_for(dx))
        s.speed = float(self.speed)
        if s.rec < 0:
            raise NotImplementedError(f"reconstruction {rec.name!r} is not on the GB300 path")
        if s.rec == L.SHK_REC_LEARNED:
            from pyshocks_gb300.learned import c_scheme_fields

            c_scheme_fields(rec, s)
        return s


# {{{ Burgers


@dataclass(frozen=True)
class BurgersScheme(GpuConservationLawScheme):
    """``src/pyshocks/burgers/schemes.py:29-34``."""


@flux.register(BurgersScheme)
def _flux_burgers(scheme, t, x, u):
    return u**2 / 2


@dataclass(frozen=True)
class Godunov(BurgersScheme):
    """Godunov (upwind) scheme, ``src/pyshocks/burgers/schemes.py:71-89``: the
    upwind flux of ``src/pyshocks/scalar.py:91-132`` with ``a = u``."""

    flux_code: ClassVar[int] = L.SHK_FLUX_GODUNOV


@dataclass(frozen=True)
class EngquistOsher(BurgersScheme):
    """Engquist-Osher scheme, ``src/pyshocks/burgers/schemes.py:160-196``:
    ``f(max(ul, w)) + f(min(ur, w)) - f(w)`` with ``w = 0`` the minimum of the
    convex Burgers flux (``src/pyshocks/scalar.py:287-322``)."""

    flux_code: ClassVar[int] = L.SHK_FLUX_EO

    @property
    def omega(self) -> float:
        return 0.0


@dataclass(frozen=True)
class Rusanov(BurgersScheme):
    """``src/pyshocks/burgers/schemes.py:98-107``."""

    alpha: float = 1.0

    def nu_for(self, dx: float) -> float:
        # scalar.py:231-234 on a uniform grid (df = dx)
        return 1.0 if abs(self.alpha - 1.0) <= 1.0e-8 else dx ** (self.alpha - 1)

    def cfl_constant(self, dx: float) -> float:
        # burgers/schemes.py:127
        return 0.5 * dx ** (2 - self.alpha)


@dataclass(frozen=True)
class LaxFriedrichs(Rusanov):
    """Global Lax-Friedrichs (``src/pyshocks/burgers/schemes.py:136-153``)."""

    flux_code: ClassVar[int] = L.SHK_FLUX_LF


@dataclass(frozen=True)
class ESWENO32(BurgersScheme):
    """Energy-stable WENO (``src/pyshocks/burgers/schemes.py:205-216``)."""

    flux_code: ClassVar[int] = L.SHK_FLUX_ESWENO

    def __post_init__(self) -> None:
        if not isinstance(self.rec, rec_mod.ESWENO32):
            raise TypeError("ESWENO32 scheme requires the ESWENO32 reconstruction.")


@bind.register(ESWENO32)
def _bind_burgers_esweno32(scheme: ESWENO32, grid: Grid, bc: Boundary) -> ESWENO32:
    """``src/pyshocks/burgers/schemes.py:219-227`` with ``es_weno_parameters``
    (``src/pyshocks/weno.py:265-281``) on ``u0 = 1``."""
    i = grid.i_
    eps = float(torch.sum(grid.dx[i].double() * 1.0)) * grid.dx_min**2
    delta = grid.dx_min**2
    return replace(scheme, rec=replace(scheme.rec, eps=eps, delta=delta))


# }}}


# {{{ linear advection and LWR traffic flow (flux plug-ins)


@dataclass(frozen=True)
class AdvectionRusanov(GpuConservationLawScheme):
    """Linear advection ``u_t + c u_x = 0`` with the Rusanov flux (for ``c > 0``
    the upwind flux of the reference's advection Godunov scheme)."""

    velocity: float = 1.0
    equation_code: ClassVar[int] = L.SHK_EQ_ADVECTION

    @property
    def speed(self) -> float:
        return float(self.velocity)

    def cfl_constant(self, dx: float) -> float:
        return 0.5 * dx


@flux.register(AdvectionRusanov)
def _flux_advection(scheme, t, x, u):
    return scheme.velocity * u


@dataclass(frozen=True)
class LWRRusanov(GpuConservationLawScheme):
    """LWR traffic flow ``rho_t + (rho (1 - rho))_x = 0`` with the Rusanov flux
    and wave speed ``1 - 2 rho``."""

    equation_code: ClassVar[int] = L.SHK_EQ_LWR


@flux.register(LWRRusanov)
def _flux_lwr(scheme, t, x, u):
    return (1 - u) * u


# }}}


# {{{ CUDA implementations of the generics


def _check_state(grid: Grid, u: torch.Tensor) -> None:
    if not (isinstance(u, torch.Tensor) and u.is_cuda):
        raise TypeError("the GB300 path expects a CUDA tensor")
    if u.dtype != torch.float64:
        raise TypeError("single-instance entry points are float64 (use BatchedSolver for float32)")
    if u.dim() != 1 or u.shape[0] != grid.x.shape[0] or not u.is_contiguous():
        raise ValueError(f"expected a contiguous array of {grid.x.shape[0]} cells")


def _check_bc(bc: Boundary) -> None:
    if isinstance(bc, PeriodicBoundary):
        return
    if isinstance(bc, TwoSidedBoundary) and all(
            isinstance(b, (DirichletBoundary, NeumannBoundary)) for b in (bc.left, bc.right)):
        return
    raise NotImplementedError(f"{type(bc).__name__} is not on the GB300 path")


def c_boundary(bc: Boundary, grid: Grid, times) -> L.ShkBoundary | None:
    """The boundary data of a call at its stage times (``None``: periodic).
    Dirichlet: ``g(t_s, x)`` at the three ghost centres of each side (the one
    next to the interior first); Neumann: ``g(t_s)``."""
    _check_bc(bc)
    if isinstance(bc, PeriodicBoundary):
        return None
    out = L.ShkBoundary()
    g, n = grid.nghosts, grid.ncells
    h = float(grid.dx_min)
    for side, b in ((0, bc.left), (1, bc.right)):
        kind = L.SHK_BC_DIRICHLET if isinstance(b, DirichletBoundary) else L.SHK_BC_NEUMANN
        if side == 0:
            out.left = kind
            idx = [g - 1 - k for k in range(min(g, 3))]
        else:
            out.right = kind
            idx = [g + n + k for k in range(min(g, 3))]
        x = grid.x[torch.tensor(idx, device=grid.x.device)].double()
        if g < 3:
            # cells beyond a grid with fewer than 3 ghosts (their values reach
            # only ghost outputs): centres continued outward
            x0 = float(grid.f[g]) if side == 0 else float(grid.f[g + n])
            sgn = -1.0 if side == 0 else 1.0
            extra = [x0 + sgn * (k + 0.5) * h for k in range(g, 3)]
            x = torch.cat([x, torch.tensor(extra, dtype=x.dtype, device=x.device)])
        for s_, ts in enumerate(times):
            if kind == L.SHK_BC_DIRICHLET:
                vals = torch.as_tensor(b.g(ts, x), dtype=torch.float64).reshape(-1).cpu()
                for k in range(3):
                    out.dirichlet[(s_ * 2 + side) * 3 + k] = float(vals[k])
            else:
                out.neumann[s_ * 2 + side] = float(b.g(ts))
    return out


def ghosted_workspace(grid: Grid, device) -> torch.Tensor:
    """Device workspace of the ghosted-array entry points
    (``shk_ghosted_workspace_bytes``; from torch's caching allocator)."""
    nb = int(L.lib().shk_ghosted_workspace_bytes(grid.ncells, grid.nghosts))
    return torch.empty(nb, dtype=torch.uint8, device=device)


def ghosted_supported(scheme) -> bool:
    """Schemes of the ghosted-array kernels: Rusanov / Lax-Friedrichs with the
    constant or WENO-JS5 reconstruction."""
    return scheme.flux_code in (L.SHK_FLUX_RUSANOV, L.SHK_FLUX_LF) and getattr(
        scheme.rec, "code", -1) in (L.SHK_REC_CONSTANT, L.SHK_REC_WENOJS53)


@apply_operator.register(GpuConservationLawScheme)
def _apply_operator_gpu(scheme, grid: Grid, bc: Boundary, t: Any, u: torch.Tensor):
    """``src/pyshocks/schemes.py:339-346`` in one kernel: periodic ghost fill,
    reconstruction, numerical flux and flux difference. The global
    Lax-Friedrichs flux (whose wave speed is the maximum over the whole
    boundary-filled array, ``scalar.py:258-278``) runs on the ghosted-array
    kernels (``shk_apply_operator_ghosted_f64``), which also give the
    reference's ghost outputs."""
    _check_bc(bc)
    _check_state(grid, u)
    lib = L.lib()
    cs = scheme.c_scheme(grid.dx_min)
    g = grid.nghosts
    n = grid.ncells
    out = torch.empty_like(u)
    stream = L.stream_handle()
    cb = c_boundary(bc, grid, (float(t),) * 3)
    bptr = None if cb is None else ctypes.byref(cb)
    if scheme.flux_code == L.SHK_FLUX_LF:
        if not ghosted_supported(scheme):
            raise NotImplementedError("global Lax-Friedrichs runs with the constant or WENO-JS5 "
                                      "reconstruction on the GB300 path")
        ws = ghosted_workspace(grid, u.device)
        L.check(lib.shk_apply_operator_ghosted_f64(cs, bptr, u.data_ptr(), out.data_ptr(), n, g,
                                                   float(grid.dx_min), ws.data_ptr(), ws.numel(),
                                                   stream), "apply_operator_ghosted")
        return out
    amax = None
    L.check(
        lib.shk_apply_operator_bc_f64(cs, bptr, u.data_ptr(), out.data_ptr(), n, g,
                                      float(grid.dx_min), L.ptr(amax), stream),
        "apply_operator",
    )
    return out


@predict_timestep.register(GpuConservationLawScheme)
def _predict_timestep_gpu(scheme, grid: Grid, bc: Boundary, t: Any, u: torch.Tensor):
    """``0.5 dx^(2-alpha) / max|f'(u_i)|`` (``src/pyshocks/burgers/schemes.py:121-127``)
    as a 0-d device tensor."""
    _check_state(grid, u)
    lib = L.lib()
    dt = torch.empty((), dtype=torch.float64, device=u.device)
    L.check(
        lib.shk_predict_timestep_f64(scheme.c_scheme(grid.dx_min), u.data_ptr(), grid.ncells, grid.nghosts,
                                     scheme.cfl_constant(grid.dx_min), 1.0, dt.data_ptr(),
                                     L.stream_handle()),
        "predict_timestep",
    )
    return dt


def ssprk33_step(scheme, grid: Grid, bc: Boundary, dt: float, u: torch.Tensor,
                 t: float = 0.0) -> torch.Tensor:
    """One fused SSPRK33 step (``src/pyshocks/timestepping.py:312-320``) from
    time *t*; a Dirichlet / Neumann boundary is applied before each stage at
    the stage times t, t + dt, t + dt/2."""
    _check_bc(bc)
    _check_state(grid, u)
    out = torch.empty_like(u)
    dt = float(dt)
    cb = c_boundary(bc, grid, (float(t), float(t) + dt, float(t) + 0.5 * dt))
    if scheme.flux_code == L.SHK_FLUX_LF:
        # the per-stage global maximum: the three stages on the ghosted-array
        # kernels (shk_ssprk33_step_ghosted_f64), no host round trip
        if not ghosted_supported(scheme):
            raise NotImplementedError("global Lax-Friedrichs runs with the constant or WENO-JS5 "
                                      "reconstruction on the GB300 path")
        ws = ghosted_workspace(grid, u.device)
        L.check(L.lib().shk_ssprk33_step_ghosted_f64(
            scheme.c_scheme(grid.dx_min), None if cb is None else ctypes.byref(cb), u.data_ptr(),
            out.data_ptr(), grid.ncells, grid.nghosts, float(grid.dx_min), dt, ws.data_ptr(),
            ws.numel(), L.stream_handle()), "ssprk33_step_ghosted")
        return out
    L.check(
        L.lib().shk_ssprk33_step_bc_f64(scheme.c_scheme(grid.dx_min),
                                        None if cb is None else ctypes.byref(cb), u.data_ptr(),
                                        out.data_ptr(), grid.ncells, grid.nghosts,
                                        float(grid.dx_min), dt, L.stream_handle()),
        "ssprk33_step",
    )
    return out


# }}}


# {{{ make_scheme_from_name


_SCHEMES: dict[str, type[SchemeBase]] = {
    "default": LaxFriedrichs,
    "godunov": Godunov,
    "rusanov": Rusanov,
    "lf": LaxFriedrichs,
    "eo": EngquistOsher,
    "esweno32": ESWENO32,
}


def scheme_ids() -> tuple[str, ...]:
    return tuple(_SCHEMES)


# the reference's entropy-stable summation-by-parts schemes (SS-MUSCL,
# SS-WENO 2-4-2, flux-split Rusanov on SBP operators): not on this path
_NOT_ON_THIS_PATH = ("ssmuscl", "ssweno242", "splitrusanov")


def make_scheme_from_name(name: str, **kwargs: Any) -> SchemeBase:
    """``src/pyshocks/burgers/__init__.py:82-98``."""
    cls = _SCHEMES.get(name)
    if cls is None:
        if name in _NOT_ON_THIS_PATH:
            raise NotImplementedError(
                f"Scheme {name!r} (summation-by-parts, entropy-stable) has no GPU "
                f"implementation. Try one of {', '.join(scheme_ids())}.")
        raise ValueError(f"Scheme {name!r} not found. Try one of {', '.join(scheme_ids())}.")
    return cls(**{f.name: kwargs[f.name] for f in fields(cls) if f.name in kwargs})


# }}}
