"""NumPy float64 restatement of pyshocks' 1D conservation-law path.

THIS IS TEST INFRASTRUCTURE (the oracle). Only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it,
and only as the checker or the timed CPU baseline. The product package
(``pyshocks_gb300``) never imports it and has no CPU fallback.

Every function restates the reference's arithmetic, in the reference's order of
operations, citing the file:line of ``alexfikl/pyshocks`` (``src/pyshocks/...``)
it follows. ``jnp.convolve(..., mode="same")`` is restated with
``numpy.convolve(..., mode="same")`` (identical definition; the summation order
inside XLA's convolution is not reproducible here and may differ in the last
bit).

Array layout follows the reference: one instance is a ghosted array of
``n + 2 g`` cell values, faces are ``n + 2 g + 1``.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Callable, Iterator

import numpy as np

# {{{ coefficients


@dataclass(frozen=True)
class Stencil:
    """WENO stencil coefficients (``src/pyshocks/weno.py:54-98``)."""

    a: np.ndarray
    b: np.ndarray
    c: np.ndarray
    d: np.ndarray


def weno_js_32_coefficients() -> Stencil:
    """Third-order WENO-JS coefficients (``src/pyshocks/weno.py:166-203``).

    Taps are ordered ``(i + 1, i, i - 1)`` so they can be fed to a convolution.
    """
    a = np.array([1.0])
    b = np.array([[[0.0, 1.0, -1.0]], [[1.0, -1.0, 0.0]]])
    c = np.array([[0.0, 3.0 / 2.0, -1.0 / 2.0], [1.0 / 2.0, 1.0 / 2.0, 0.0]])
    d = np.array([[1.0 / 3.0, 2.0 / 3.0]]).T
    return Stencil(a=a, b=b, c=c, d=d)


def weno_js_53_coefficients() -> Stencil:
    """Fifth-order WENO-JS coefficients (``src/pyshocks/weno.py:206-244``).

    Taps are ordered ``(i + 2, i + 1, i, i - 1, i - 2)``.
    """
    a = np.array([13.0 / 12.0, 1.0 / 4.0])
    b = np.array(
        [
            [[0.0, 0.0, 1.0, -2.0, 1.0], [0.0, 0.0, 3.0, -4.0, 1.0]],
            [[0.0, 1.0, -2.0, 1.0, 0.0], [0.0, 1.0, 0.0, -1.0, 0.0]],
            [[1.0, -2.0, 1.0, 0.0, 0.0], [1.0, -4.0, 3.0, 0.0, 0.0]],
        ]
    )
    c = np.array(
        [
            [0.0, 0.0, 11.0 / 6.0, -7.0 / 6.0, 2.0 / 6.0],
            [0.0, 2.0 / 6.0, 5.0 / 6.0, -1.0 / 6.0, 0.0],
            [-1.0 / 6.0, 5.0 / 6.0, 2.0 / 6.0, 0.0, 0.0],
        ]
    )
    d = np.array([[1.0 / 10.0, 6.0 / 10.0, 3.0 / 10.0]]).T
    return Stencil(a=a, b=b, c=c, d=d)


# }}}


# {{{ weno


def convolve1d(u: np.ndarray, w: np.ndarray) -> np.ndarray:
    """``convolve1d(..., mode=Same)`` (``src/pyshocks/convolve.py:113-114``):
    a zero-padded "same" convolution."""
    return np.convolve(u, w, mode="same")


def weno_smoothness(s: Stencil, u: np.ndarray) -> np.ndarray:
    """Smoothness indicators (``src/pyshocks/weno.py:114-140``)."""
    return np.stack([
        sum(s.a[j] * convolve1d(u, s.b[i, j, :]) ** 2 for j in range(s.a.size))
        for i in range(s.b.shape[0])
    ])


def weno_interp(s: Stencil, u: np.ndarray) -> np.ndarray:
    """Sub-stencil interpolants (``src/pyshocks/weno.py:143-157``)."""
    return np.stack([convolve1d(u, s.c[i, :]) for i in range(s.c.shape[0])])


def weno_js_weights(s: Stencil, u: np.ndarray, eps: float) -> np.ndarray:
    """WENO-JS nonlinear weights (``src/pyshocks/weno.py:247-256``)."""
    beta = weno_smoothness(s, u)
    alpha = s.d / (eps + beta) ** 2
    return alpha / np.sum(alpha, axis=0, keepdims=True)


def es_weno_weights(s: Stencil, u: np.ndarray, eps: float) -> np.ndarray:
    """ES-WENO weights (``src/pyshocks/weno.py:284-296``)."""
    beta = weno_smoothness(s, u)
    tau = np.pad((u[2:] - 2 * u[1:-1] + u[:-2]) ** 2, 1)
    alpha = s.d * (1 + tau / (eps + beta))
    return alpha / np.sum(alpha, axis=0, keepdims=True)


def es_weno_parameters(grid: "CellGrid", u0: np.ndarray) -> tuple[float, float]:
    """ES-WENO ``(eps, delta)`` (``src/pyshocks/weno.py:265-281``):
    ``eps = sum(dx |u0|) dx_min^2`` over the interior, ``delta = dx_min^2``.
    The Burgers ES-WENO scheme binds them with ``u0 = 1``
    (``src/pyshocks/burgers/schemes.py:219-227``)."""
    i = grid.i_
    eps = np.sum(grid.dx[i] * np.abs(u0[i])) * grid.dx_min**2
    delta = grid.dx_min**2
    return float(eps), float(delta)


# }}}


# {{{ reconstruction


def _reconstruct_weno_js_side(s: Stencil, eps: float, f: np.ndarray) -> np.ndarray:
    """``src/pyshocks/reconstruction.py:351-355``."""
    omega = weno_js_weights(s, f, eps)
    uhat = weno_interp(s, f)
    return np.sum(omega * uhat, axis=0)


def reconstruct_wenojs(
    s: Stencil, eps: float, f: np.ndarray
) -> tuple[np.ndarray, np.ndarray]:
    """``(ul, ur)`` face values (``src/pyshocks/reconstruction.py:358-377``)."""
    ur = _reconstruct_weno_js_side(s, eps, f)
    ul = _reconstruct_weno_js_side(s, eps, f[::-1])[::-1]
    return ul, ur


def _reconstruct_es_weno_side(s: Stencil, eps: float, f: np.ndarray) -> np.ndarray:
    """``src/pyshocks/reconstruction.py:413-417``."""
    omega = es_weno_weights(s, f, eps)
    uhat = weno_interp(s, f)
    return np.sum(omega * uhat, axis=0)


# {{{ MUSCL (src/pyshocks/limiters.py, src/pyshocks/reconstruction.py:172-296)

LIMITERS = ("none", "minmod", "mc", "superbee", "vanalbada", "vanleer", "koren")
#: limiters with phi(1/r) = phi(r)/r (limiters.py: is_symmetric)
SYMMETRIC = {"minmod", "mc", "superbee", "vanleer"}


def limiter_phi(name: str, r: np.ndarray, param: float = 1.0) -> np.ndarray:
    """``evaluate(lm, r)`` (``limiters.py:137-139,194-198,229-231,265-267,
    316-323,359-362,386-388``); *param* is theta (minmod) or the van Albada
    variant."""
    if name == "none":
        return np.ones_like(r)
    if name == "minmod":
        return np.maximum(0.0, np.minimum(np.minimum(param, param * r), (1 + r) / 2))
    if name == "mc":
        return np.maximum(0.0, np.minimum(np.minimum(2, 2 * r), (1 + r) / 2))
    if name == "superbee":
        return np.maximum(0.0, np.maximum(np.minimum(1, 2 * r), np.minimum(2, r)))
    if name == "vanalbada":
        phi = (r**2 + r) / (r**2 + 1) if int(param) == 1 else 2 * r / (r**2 + 1)
        return np.maximum(0.0, phi)
    if name == "vanleer":
        rabs = np.abs(r)
        return np.maximum(0.0, (r + rabs) / (1 + rabs))
    if name == "koren":
        return np.maximum(0.0, np.minimum(np.minimum(2, 2 * r), (1 + 2 * r) / 3))
    raise ValueError(name)


def is_symmetric(name: str, param: float = 1.0) -> bool:
    return name in SYMMETRIC or (name == "vanalbada" and int(param) == 1)


def local_slope_ratio(u: np.ndarray, atol: float = 1.0e-12) -> np.ndarray:
    """``limiters.py:110-125``."""
    sl = u[1:-1] - u[:-2]
    sr = u[2:] - u[1:-1]
    mask = (np.abs(sr) < atol).astype(u.dtype)
    sl = np.where(mask, 0.0, sl)
    sr = np.where(mask, 1.0, sr)
    return sl / sr


def reconstruct_muscl(name: str, param: float, atol: float, f: np.ndarray,
                      u: np.ndarray | None = None):
    """``(ul, ur)`` of the flux-limited MUSCL reconstruction
    (``reconstruction.py:212-245``); the limiter works on *u* (default *f*)."""
    u = f if u is None else u
    r = np.pad(local_slope_ratio(u, atol=atol), 1)
    phi_r = limiter_phi(name, r, param)
    if is_symmetric(name, param):
        with np.errstate(divide="ignore", invalid="ignore"):
            phi_inv_r = np.where(np.abs(r) < atol, 0.0, phi_r / r)
    else:
        with np.errstate(divide="ignore"):
            inv_r = np.where(np.abs(r) < atol, atol, 1 / r)
        phi_inv_r = limiter_phi(name, inv_r, param)
    ur = np.pad(f[:-1] + 0.5 * phi_r[:-1] * (f[1:] - f[:-1]), (0, 1))
    ul = np.pad(f[1:] - 0.5 * phi_inv_r[1:] * (f[1:] - f[:-1]), (1, 0))
    return ul, ur


def _minmod(a, b):
    return np.where(a * b < 0.0, 0.0, np.where(np.abs(a) < np.abs(b), a, b))


def slope_limit(name: str, param: float, x: np.ndarray, u: np.ndarray) -> np.ndarray:
    """``slope_limit(lm, grid, u)`` (``limiters.py:147-155,201-209,234-245,
    270-278,326-339,365-375``); Koren has no slope form in the reference."""
    sl = (u[1:-1] - u[:-2]) / (x[1:-1] - x[:-2])
    sr = (u[2:] - u[1:-1]) / (x[2:] - x[1:-1])
    if name == "none":
        # the reference's unlimited slope adds the neighbours (limiters.py:150)
        s = (u[2:] + u[:-2]) / (x[2:] - x[:-2])
    elif name == "minmod":
        s = _minmod(sl, sr)
    elif name == "mc":
        sc = (u[2:] - u[:-2]) / (x[2:] - x[:-2])
        s = _minmod(_minmod(sl, sr), sc)
    elif name == "superbee":
        s = np.maximum(_minmod(sl, 2 * sr), _minmod(2 * sl, sr))
    elif name == "vanalbada":
        with np.errstate(divide="ignore", invalid="ignore"):
            if int(param) == 1:
                s = np.where(sl * sr <= 0.0, 0.0, sl * sr * (sl + sr) / (sl**2 + sr**2))
            else:
                s = np.where(sl * sr <= 0.0, 0.0, 2.0 * sl * sr / (sl**2 + sr**2))
    elif name == "vanleer":
        with np.errstate(divide="ignore", invalid="ignore"):
            s = np.where(sl * sr <= 0.0, 0.0, 2.0 * sl * sr / (sl + sr))
    else:
        raise NotImplementedError(name)
    return np.pad(s, 1)


def reconstruct_muscls(name: str, param: float, x: np.ndarray, dx: float, f: np.ndarray):
    """``(ul, ur)`` of the slope-limited MUSCL reconstruction
    (``reconstruction.py:271-290``)."""
    du = slope_limit(name, param, x, f)
    return f - 0.5 * dx * du, f + 0.5 * dx * du


# }}}


def reconstruct_esweno32(
    s: Stencil, eps: float, f: np.ndarray
) -> tuple[np.ndarray, np.ndarray]:
    """``src/pyshocks/reconstruction.py:420-439``."""
    ur = _reconstruct_es_weno_side(s, eps, f)
    ul = _reconstruct_es_weno_side(s, eps, f[::-1])[::-1]
    return ul, ur


# }}}


# {{{ grid / boundary


@dataclass(frozen=True)
class CellGrid:
    """Uniform cell grid (``src/pyshocks/grid.py:131-179``)."""

    a: float
    b: float
    n: int
    nghosts: int
    x: np.ndarray
    f: np.ndarray
    dx: np.ndarray
    dx_min: float

    @property
    def i_(self) -> slice:
        """Interior slice (``src/pyshocks/grid.py:84-86``)."""
        return np.s_[self.nghosts : self.x.size - self.nghosts]


def make_uniform_cell_grid(a: float, b: float, n: int, nghosts: int = 3) -> CellGrid:
    """``src/pyshocks/grid.py:131-179``."""
    h = (b - a) / n
    f = np.linspace(a - nghosts * h, b + nghosts * h, n + 2 * nghosts + 1)
    x = (f[1:] + f[:-1]) / 2
    dx = np.full_like(x, h)
    return CellGrid(a=a, b=b, n=n, nghosts=nghosts, x=x, f=f, dx=dx, dx_min=h)


def apply_boundary_periodic(u: np.ndarray, g: int) -> np.ndarray:
    """Periodic ghost fill (``src/pyshocks/scalar.py:529-540``): the right
    ghosts first, then the left ghosts."""
    u = u.copy()
    n = u.size
    u[n - g :] = u[g : 2 * g]
    u[:g] = u[n - 2 * g : n - g]
    return u


def apply_boundary_dirichlet(u: np.ndarray, grid: "CellGrid", t: float, ga: Callable,
                             gb: Callable) -> np.ndarray:
    """Dirichlet ghost fill (``src/pyshocks/scalar.py:419-429``): the ghost
    cells of each side take ``g(t, x)`` at their centres (left, then right,
    as ``TwoSidedBoundary`` applies them, ``scalar.py:373-382``)."""
    u = u.copy()
    g = grid.nghosts
    u[:g] = ga(t, grid.x[:g])
    u[u.size - g:] = gb(t, grid.x[u.size - g:])
    return u


def apply_boundary_neumann(u: np.ndarray, grid: "CellGrid", t: float, ga: Callable,
                           gb: Callable) -> np.ndarray:
    """Neumann ghost fill (``src/pyshocks/scalar.py:469-495``): ghost cells
    mirrored about the boundary face, ``u_from + side (x_from - x_to) g(t)``."""
    u = u.copy()
    g = grid.nghosts
    n = u.size
    for side, fn in ((-1, ga), (+1, gb)):
        if side == -1:
            ifrom = np.arange(g, 2 * g)
            ito = np.arange(g - 1, -1, -1)
        else:
            ifrom = np.arange(n - 2 * g, n - g)
            ito = np.arange(n - 1, n - g - 1, -1)
        u[ito] = u[ifrom] + side * (grid.x[ifrom] - grid.x[ito]) * fn(t)
    return u


# }}}


# {{{ fluxes


def flux_burgers(u: np.ndarray) -> np.ndarray:
    """``src/pyshocks/burgers/schemes.py:37-39``."""
    return u**2 / 2


def flux_linear_advection(u: np.ndarray, speed: float = 1.0) -> np.ndarray:
    """Linear advection flux ``a u``."""
    return speed * u


def flux_lwr(u: np.ndarray) -> np.ndarray:
    """LWR traffic flux ``rho (1 - rho)`` (the flux plug-in pattern of
    ``examples/traffic-flow-model.py:14-39``)."""
    return u * (1 - u)


def wavespeed_burgers(u: np.ndarray) -> np.ndarray:
    """``f'(u) = u``: Burgers passes ``a = u`` (``src/pyshocks/burgers/schemes.py:116-118``)."""
    return u


def wavespeed_linear_advection(u: np.ndarray, speed: float = 1.0) -> np.ndarray:
    return np.full_like(u, speed)


def wavespeed_lwr(u: np.ndarray) -> np.ndarray:
    return 1 - 2 * u


FLUXES: dict[str, tuple[Callable, Callable]] = {
    "burgers": (flux_burgers, wavespeed_burgers),
    "advection": (flux_linear_advection, wavespeed_linear_advection),
    "lwr": (flux_lwr, wavespeed_lwr),
}


def scalar_flux_rusanov(
    ul: np.ndarray,
    ur: np.ndarray,
    a: np.ndarray | float,
    flux: Callable,
    nu: float = 1.0,
) -> np.ndarray:
    """Rusanov / local Lax-Friedrichs flux (``src/pyshocks/scalar.py:192-249``).

    *a* is the cell wave speed array (local) or a scalar (global); the local
    speed at a face is ``max(|a_i|, |a_{i+1}|)`` of the *cell* values
    (``scalar.py:243-246``).
    """
    fl = flux(ul)
    fr = flux(ur)
    a = np.abs(a)
    if isinstance(a, np.ndarray) and a.size == ul.size:
        a = np.maximum(a[1:], a[:-1])
    fnum = 0.5 * (fl[1:] + fr[:-1]) - 0.5 * a * nu * (ul[1:] - ur[:-1])
    return np.pad(fnum, 1)


def scalar_flux_upwind(
    ul: np.ndarray, ur: np.ndarray, al: np.ndarray, ar: np.ndarray, flux: Callable
) -> np.ndarray:
    """Upwind flux (``src/pyshocks/scalar.py:91-132``)."""
    fl = flux(ul)
    fr = flux(ur)
    aavg = (ar[:-1] + al[1:]) / 2
    fnum = np.where(aavg > 0, fr[:-1], fl[1:])
    return np.pad(fnum, 1)


# }}}


# {{{ schemes


@dataclass(frozen=True)
class SchemeSpec:
    """A plain description of a scheme on the hot path.

    * ``flux_kind``: ``"rusanov"`` (``burgers/schemes.py:110-118``),
      ``"lf"`` (``burgers/schemes.py:145-153``), ``"esweno"``
      (``burgers/schemes.py:230-256``), ``"godunov"`` (``burgers/schemes.py:83-89``)
      or ``"eo"`` (``burgers/schemes.py:188-196``).
    * ``rec``: ``"wenojs53"``, ``"wenojs32"``, ``"esweno32"`` or ``"constant"``
      (``reconstruction.py:153-163``).
    * ``equation``: ``"burgers"``, ``"advection"`` or ``"lwr"``.
    """

    flux_kind: str = "rusanov"
    rec: str = "wenojs53"
    eps: float = 1.0e-6
    delta: float = 1.0e-6
    alpha: float = 1.0
    equation: str = "burgers"
    #: MUSCL / MUSCLS (``rec="muscl"`` / ``"muscls"``): limiter name, its
    #: parameter (theta or variant), the slope cut atol and the grid
    limiter: str = "minmod"
    limiter_param: float = 1.0
    atol: float = 1.0e-12
    x: Any = None
    dx: float = 0.0

    @property
    def stencil(self) -> Stencil:
        if self.rec == "wenojs53":
            return weno_js_53_coefficients()
        return weno_js_32_coefficients()


def reconstruct(spec: SchemeSpec, f: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    if spec.rec == "constant":
        return f, f
    if spec.rec == "muscl":
        return reconstruct_muscl(spec.limiter, spec.limiter_param, spec.atol, f)
    if spec.rec == "muscls":
        return reconstruct_muscls(spec.limiter, spec.limiter_param, spec.x, spec.dx, f)
    if spec.rec == "esweno32":
        return reconstruct_esweno32(spec.stencil, spec.eps, f)
    return reconstruct_wenojs(spec.stencil, spec.eps, f)


def numerical_flux(spec: SchemeSpec, grid: CellGrid, u: np.ndarray) -> np.ndarray:
    """``numerical_flux`` for the registered schemes on the hot path."""
    flux, speed = FLUXES[spec.equation]
    if spec.flux_kind in {"rusanov", "lf"}:
        # artificial viscosity (scalar.py:230-234)
        if abs(spec.alpha - 1.0) > 1.0e-8:
            df = np.diff(grid.x)
            nu = df ** (spec.alpha - 1)
        else:
            nu = 1.0
        ul, ur = reconstruct(spec, u)
        a = speed(u)
        if spec.flux_kind == "lf":
            # global maximum over the whole ghosted array (scalar.py:277)
            a = np.max(np.abs(a))
        return scalar_flux_rusanov(ul, ur, a, flux, nu)
    if spec.flux_kind == "godunov":
        ul, ur = reconstruct(spec, u)
        a = speed(u)
        al, ar = reconstruct(spec, a)
        return scalar_flux_upwind(ul, ur, al, ar, flux)
    if spec.flux_kind == "eo":
        # scalar.py:287-322 with omega = 0 (burgers/schemes.py:184-196)
        ul, ur = reconstruct(spec, u)
        omega = 0.0
        fr = flux(np.maximum(ur, omega))
        fl = flux(np.minimum(ul, omega))
        fomega = flux(np.full(u.size - 1, omega))
        return np.pad(fr[:-1] + fl[1:] - fomega, 1)
    if spec.flux_kind == "esweno":
        # burgers/schemes.py:230-256
        s = weno_js_32_coefficients()
        omega = es_weno_weights(s, u, spec.eps)[0, :]
        mu = np.sqrt((omega[1:] - omega[:-1]) ** 2 + spec.delta**2) / 8.0
        gnum = -(mu + (omega[1:] - omega[:-1]) / 8.0) * (u[1:] - u[:-1])
        gnum = np.pad(gnum, 1)
        ul, ur = reconstruct(spec, u)
        fnum = scalar_flux_upwind(ul, ur, ul, ur, flux)
        return fnum + gnum
    raise ValueError(f"unknown flux kind: {spec.flux_kind!r}")


def apply_operator(spec: SchemeSpec, grid: CellGrid, u: np.ndarray, t: float = 0.0,
                   bc: Callable | None = None) -> np.ndarray:
    """``src/pyshocks/schemes.py:339-346``; *bc* ``(t, u) -> u`` fills the
    ghost cells (periodic by default)."""
    u = apply_boundary_periodic(u, grid.nghosts) if bc is None else bc(t, u)
    f = numerical_flux(spec, grid, u)
    return -(f[1:] - f[:-1]) / grid.dx


def predict_timestep(spec: SchemeSpec, grid: CellGrid, u: np.ndarray) -> float:
    """CFL estimate.

    * Rusanov / LF: ``0.5 dx^(2 - alpha) / max|u|``
      (``src/pyshocks/burgers/schemes.py:121-127``);
    * other Burgers schemes: ``0.5 dx / max|u|`` (``burgers/schemes.py:42-49``);
    * LWR: ``0.5 dx / max|1 - 2 rho|`` (wave speed of the LWR flux).
    """
    _, speed = FLUXES[spec.equation]
    smax = np.max(np.abs(speed(u[grid.i_])))
    if spec.flux_kind in {"rusanov", "lf"}:
        return 0.5 * grid.dx_min ** (2 - spec.alpha) / smax
    return 0.5 * grid.dx_min / smax


# }}}


# {{{ time stepping


def ssprk33(
    source: Callable[[float, np.ndarray], np.ndarray],
    dt: float,
    t: float,
    u: np.ndarray,
) -> np.ndarray:
    """``src/pyshocks/timestepping.py:312-320``."""
    fn = source
    k1 = u + dt * fn(t, u)
    k2 = 3.0 / 4.0 * u + 1.0 / 4.0 * (k1 + dt * fn(t + dt, k1))
    return 1.0 / 3.0 * u + 2.0 / 3.0 * (k2 + dt * fn(t + 0.5 * dt, k2))


@dataclass(frozen=True)
class StepCompleted:
    """``src/pyshocks/timestepping.py:46-65``."""

    t: float
    tfinal: float
    dt: float
    iteration: int
    u: np.ndarray


def step(
    predict: Callable[[float, np.ndarray], float],
    source: Callable[[float, np.ndarray], np.ndarray],
    u0: np.ndarray,
    *,
    maxit: int | None = None,
    tstart: float = 0.0,
    tfinal: float | None = None,
) -> Iterator[StepCompleted]:
    """``src/pyshocks/timestepping.py:89-152`` (SSPRK33 stepper, no checkpoint)."""
    dtype = u0.dtype.type
    if tfinal is None:
        tfinal = float(np.finfo(u0.dtype).max)
    m = 0
    t = dtype(tstart)
    tfinal = dtype(tfinal)
    u = u0
    yield StepCompleted(t=t, tfinal=tfinal, dt=dtype(0.0), iteration=m, u=u)
    while True:
        if t >= tfinal:
            break
        if maxit is not None and m >= maxit:
            break
        dt = dtype(predict(t, u))
        if tfinal != np.inf:
            dt_min = tfinal - t
            dt = dtype((dt if dt < dt_min else dt_min) + 1.0e-15)
        if not np.isfinite(dt):
            raise ValueError(f"Time step is not finite: {dt!r}.")
        u = ssprk33(source, dt, t, u)
        m += 1
        t = dtype(t + dt)
        yield StepCompleted(t=t, tfinal=tfinal, dt=dt, iteration=m, u=u)


def evolve(
    spec: SchemeSpec,
    grid: CellGrid,
    u0: np.ndarray,
    *,
    theta: float = 1.0,
    maxit: int | None = None,
    tfinal: float | None = None,
    bc: Callable | None = None,
) -> tuple[np.ndarray, list[float]]:
    """Run :func:`step` with the driver closures of ``examples/burgers.py:161-178``
    (``dt = theta * predict_timestep``); return the final state and the
    sequence of time steps taken."""

    def _predict(t, u):
        return theta * predict_timestep(spec, grid, u)

    def _source(t, u):
        return apply_operator(spec, grid, u, t, bc)

    dts = []
    event = None
    for event in step(_predict, _source, u0, maxit=maxit, tfinal=tfinal):
        if event.iteration > 0:
            dts.append(float(event.dt))
    assert event is not None
    return event.u, dts


# }}}


# {{{ norms


def norm(grid: CellGrid, u: np.ndarray, p: float | str = 1, weighted: bool = False):
    """Interior norm (``src/pyshocks/grid.py:444-506``)."""
    v = np.abs(u[grid.i_])
    dx = grid.dx[grid.i_] if weighted else 1.0
    if p == 1:
        return np.sum(v * dx)
    if p == 2:
        return np.sqrt(np.sum(v**2 * dx))
    if p in {np.inf, "inf"}:
        return np.max(v)
    if p in {-np.inf, "-inf"}:
        return np.min(v)
    if p == "tvd":
        return np.sum(np.abs(np.diff(v)))
    raise ValueError(f"Unrecognized norm order 'p': {p!r}.")


def rnorm(grid, u, v, p=1, weighted=False, atol=1.0e-14):
    """``src/pyshocks/grid.py:509-531``."""
    vnorm = norm(grid, v, p=p, weighted=weighted)
    if vnorm < atol:
        vnorm = 1.0
    return norm(grid, u - v, p=p, weighted=weighted) / vnorm


# }}}


# {{{ initial conditions (synthetic workloads)


def exact_cell_average_sine(grid: CellGrid, mean: float = 0.5) -> np.ndarray:
    """Exact cell averages of ``mean + sin(pi x)`` on every cell (ghosts
    included): ``mean + (cos(pi f_i) - cos(pi f_{i+1})) / (pi h)``."""
    f = grid.f
    h = grid.dx_min
    return mean + (np.cos(np.pi * f[:-1]) - np.cos(np.pi * f[1:])) / (np.pi * h)


def random_fourier_ic(
    rng: np.random.Generator,
    f: np.ndarray,
    *,
    nmodes: int = 8,
    njumps_max: int = 3,
    mean_range: float = 0.5,
    jump_height: float = 1.0,
) -> np.ndarray:
    """Exact cell averages on faces *f* (periodic on [-1, 1]) of
    ``m + sum_k A_k sin(k pi x + phi_k) + sum_j h_j 1[x > x_j]`` with
    ``m ~ U(-mean_range, mean_range)``, ``A_k ~ N(0, 1) / k^2``,
    ``phi_k ~ U(0, 2 pi)``, ``J ~ U{0..njumps_max}`` jumps of height
    ``U(-jump_height, jump_height)`` at ``x_j ~ U(-1, 1)``."""
    m = rng.uniform(-mean_range, mean_range)
    k = np.arange(1, nmodes + 1)
    amp = rng.normal(0.0, 1.0, size=nmodes) / k**2
    phi = rng.uniform(0.0, 2.0 * np.pi, size=nmodes)
    njumps = int(rng.integers(0, njumps_max + 1))
    heights = rng.uniform(-jump_height, jump_height, size=njumps)
    xj = rng.uniform(-1.0, 1.0, size=njumps)

    fl = f[:-1]
    fr = f[1:]
    h = fr - fl
    u = np.full(fl.shape, m, dtype=np.float64)
    for kk, ak, pk in zip(k, amp, phi):
        # exact average of sin(k pi x + phi) over [fl, fr]
        u += ak * (np.cos(kk * np.pi * fl + pk) - np.cos(kk * np.pi * fr + pk)) / (
            kk * np.pi * h
        )
    for hj, xjj in zip(heights, xj):
        # average of the Heaviside 1[x > x_j]
        frac = np.clip((fr - xjj) / h, 0.0, 1.0)
        u += hj * frac
    return u


def lwr_ic(
    rng: np.random.Generator,
    f: np.ndarray,
    *,
    nmodes: int = 8,
    nplateaus: int = 2,
    plateau: float = 0.95,
) -> np.ndarray:
    """LWR density on faces *f*: exact cell averages of
    ``0.5 + 0.3 sum_k A_k sin(k pi x + phi_k)`` (``A_k ~ N(0, 1) / k^2``),
    overwritten on *nplateaus* jam intervals (centre ``U(-1, 1)``, width
    ``U(0.05, 0.2)``, periodic) by ``plateau`` in proportion to the overlap,
    then clipped to ``[0, 1]``."""
    k = np.arange(1, nmodes + 1)
    amp = rng.normal(0.0, 1.0, size=nmodes) / k**2
    phi = rng.uniform(0.0, 2.0 * np.pi, size=nmodes)
    centres = rng.uniform(-1.0, 1.0, size=nplateaus)
    widths = rng.uniform(0.05, 0.2, size=nplateaus)

    fl = f[:-1]
    fr = f[1:]
    h = fr - fl
    base = np.zeros(fl.shape, dtype=np.float64)
    for kk, ak, pk in zip(k, amp, phi):
        base += ak * (np.cos(kk * np.pi * fl + pk) - np.cos(kk * np.pi * fr + pk)) / (
            kk * np.pi * h
        )
    rho = 0.5 + 0.3 * base
    for c, w in zip(centres, widths):
        frac = np.zeros_like(rho)
        for shift in (-2.0, 0.0, 2.0):
            lo = c - w / 2 + shift
            hi = c + w / 2 + shift
            frac += np.clip((np.minimum(fr, hi) - np.maximum(fl, lo)) / h, 0.0, 1.0)
        frac = np.minimum(frac, 1.0)
        rho = (1.0 - frac) * rho + frac * plateau
    return np.clip(rho, 0.0, 1.0)


# }}}


# {{{ quadrature / convergence helpers


def cell_average_leggauss(grid: CellGrid, func: Callable, order: int) -> np.ndarray:
    """Gauss-Legendre cell averages on every cell
    (``src/pyshocks/grid.py:393-435``)."""
    from numpy.polynomial.legendre import leggauss

    xi, wi = leggauss(order)
    xi = xi.reshape(-1, 1)
    wi = wi.reshape(-1, 1)
    f = grid.f
    dx = f[1:] - f[:-1]
    dxm = 0.5 * dx.reshape(1, -1)
    xm = 0.5 * (f[1:] + f[:-1]).reshape(1, -1)
    xim = xm + dxm * xi
    wim = dxm * wi
    return np.sum(func(xim) * wim, axis=0) / dx


def ic_sine_sine(grid: CellGrid, x: np.ndarray, k1: float = 2, k2: float = 2):
    """``src/pyshocks/funcs.py:122-137``."""
    xm = (grid.b + grid.a) / 2
    x = (x - xm) / (grid.b - grid.a)
    return np.sin(k1 * np.pi * x + np.sin(k2 * np.pi * x) / np.pi)


def estimate_order_of_convergence(h: np.ndarray, error: np.ndarray) -> float:
    """Least-squares slope of ``log(error)`` against ``log(h)``
    (``src/pyshocks/tools.py:184-262``)."""
    eoc, _ = np.polyfit(np.log10(h), np.log10(error), 1)
    return float(eoc)


# }}}

