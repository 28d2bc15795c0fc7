"""Time integration (mirrors ``src/pyshocks/timestepping.py``).

``step`` keeps the reference's generator semantics (per-step CFL dt, final-time
clip, ``+1e-15``, non-finite check). When the stepper's closures are the ones
built by :func:`make_time_stepper`, ``advance`` runs the fused three-stage
SSPRK33 kernel; arbitrary user closures take the generic three-call path.
The batched hot path (thousands of instances, no host round trip per step) is
:class:`pyshocks_gb300.batched.BatchedSolver`.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from functools import singledispatch
from typing import Any, Callable, Iterator

import numpy as np
import torch

from pyshocks_gb300.checkpointing import Checkpoint, load, save


@dataclass(frozen=True)
class StepCompleted:
    """``src/pyshocks/timestepping.py:46-65``."""

    t: float
    tfinal: float
    dt: float
    iteration: int
    u: torch.Tensor

    def __str__(self) -> str:
        return f"[{self.iteration:5d}] t = {self.t:.5e} / {self.tfinal:.5e} dt {self.dt:.5e}"


@dataclass(frozen=True)
class AdjointStepCompleted(StepCompleted):
    """``src/pyshocks/timestepping.py:68-71``."""

    p: torch.Tensor


@dataclass(frozen=True)
class Stepper:
    """``src/pyshocks/timestepping.py:74-86``."""

    predict_timestep: Callable[[Any, torch.Tensor], Any]
    source: Callable[[Any, torch.Tensor], torch.Tensor]
    checkpoint: Checkpoint | None


@dataclass(frozen=True)
class ForwardEuler(Stepper):
    """``src/pyshocks/timestepping.py:289-298``."""


@dataclass(frozen=True)
class SSPRK33(Stepper):
    """``src/pyshocks/timestepping.py:307-320``."""


# {{{ closures bound to a scheme (fused-kernel fast path)


@dataclass(frozen=True)
class OperatorSource:
    """``source(t, u) = apply_operator(scheme, grid, bc, t, u)`` (the closure of
    ``examples/burgers.py:164-165``), recognised by :func:`advance`."""

    scheme: Any
    grid: Any
    bc: Any

    def __call__(self, t, u):
        from pyshocks_gb300.schemes import apply_operator

        return apply_operator(self.scheme, self.grid, self.bc, t, u)


@dataclass(frozen=True)
class TimestepPredictor:
    """``theta * predict_timestep(scheme, grid, bc, t, u)`` (``examples/burgers.py:161-162``)."""

    scheme: Any
    grid: Any
    bc: Any
    theta: float = 1.0

    def __call__(self, t, u):
        from pyshocks_gb300.schemes import predict_timestep

        return self.theta * predict_timestep(self.scheme, self.grid, self.bc, t, u)


def make_time_stepper(scheme, grid, bc, *, theta: float = 1.0,
                      checkpoint: Checkpoint | None = None) -> SSPRK33:
    """SSPRK33 stepper with the driver closures of ``drivers/burgers-adjoint.py:48-65``."""
    return SSPRK33(
        predict_timestep=TimestepPredictor(scheme, grid, bc, theta),
        source=OperatorSource(scheme, grid, bc),
        checkpoint=checkpoint,
    )


# }}}


def _as_float(x) -> float:
    return float(x.item()) if isinstance(x, torch.Tensor) else float(x)


def step(
    stepper: Stepper,
    u0: torch.Tensor,
    *,
    maxit: int | None = None,
    tstart: float = 0.0,
    tfinal: float | None = None,
) -> Iterator[StepCompleted]:
    """``src/pyshocks/timestepping.py:89-152``. Time and time step are host
    doubles (the reference's are float64 scalars): one device-to-host read of
    ``dt`` per step, as in the reference."""
    if tfinal is None:
        tfinal = float(torch.finfo(u0.dtype).max)
    m = 0
    t = float(tstart)
    tfinal = float(tfinal)
    u = u0
    yield StepCompleted(t=t, tfinal=tfinal, dt=0.0, iteration=m, u=u)
    while True:
        if stepper.checkpoint is not None:
            save(stepper.checkpoint, m, {"m": m, "t": t, "u": u})
        if t >= tfinal:
            break
        if maxit is not None and m >= maxit:
            break
        dt = _as_float(stepper.predict_timestep(t, u))
        if tfinal != math.inf:
            dt_min = tfinal - t
            dt = (dt if dt < dt_min else dt_min) + 1.0e-15
        if not np.isfinite(dt):
            raise ValueError(f"Time step is not finite: {dt!r}.")
        u = advance(stepper, dt, t, u)
        m += 1
        t += dt
        yield StepCompleted(t=t, tfinal=tfinal, dt=dt, iteration=m, u=u)


@singledispatch
def advance(stepper: Stepper, dt: float, t: float, u: torch.Tensor) -> torch.Tensor:
    """``src/pyshocks/timestepping.py:218-233``."""
    raise NotImplementedError(type(stepper).__name__)


@advance.register(ForwardEuler)
def _advance_forward_euler(stepper, dt, t, u):
    return u + dt * stepper.source(t, u)


@advance.register(SSPRK33)
def _advance_ssprk33(stepper, dt, t, u):
    """``src/pyshocks/timestepping.py:312-320``; one library call when the
    source is an :class:`OperatorSource` of a scheme on the GB300 path (one
    fused kernel, or for the global Lax-Friedrichs flux the three stages on the
    ghosted-array kernels)."""
    src = stepper.source
    if isinstance(src, OperatorSource):
        from pyshocks_gb300 import burgers

        if isinstance(src.scheme, burgers.GpuConservationLawScheme) and (
            src.scheme.flux_code != burgers.L.SHK_FLUX_LF or burgers.ghosted_supported(src.scheme)
        ):
            return burgers.ssprk33_step(src.scheme, src.grid, src.bc, dt, u, t=float(t))
    fn = src
    k1 = u + dt * fn(t, u)
    k2 = 3.0 / 4.0 * u + 1.0 / 4.0 * (k1 + dt * fn(t + dt, k1))
    return 1.0 / 3.0 * u + 2.0 / 3.0 * (k2 + dt * fn(t + 0.5 * dt, k2))


def predict_timestep_from_maxit(tfinal: float, maxit: int) -> tuple[int, float]:
    """``src/pyshocks/timestepping.py:242-248``."""
    return maxit, tfinal / maxit + 1.0e-15


def predict_timestep_from_resolutions(a: float, b: float, resolutions, *, umax: float = 1.0,
                                      p: int = 1) -> float:
    """``src/pyshocks/timestepping.py:264-280``: a step stable for every
    resolution of a study, ``(dx_min)^p / umax`` with ``dx_min = (b - a) /
    max(resolutions)``."""
    dx = (b - a) / max(resolutions)
    return dx**p / umax


def predict_maxit_from_timestep(tfinal: float, dt: float) -> tuple[int, float]:
    """``src/pyshocks/timestepping.py:251-261``."""
    maxit = int(tfinal / dt)
    return maxit, tfinal / maxit + 1.0e-15


def adjoint_step(
    stepper: Stepper,
    p0: torch.Tensor,
    *,
    maxit: int,
    apply_boundary: Callable[[float, torch.Tensor, torch.Tensor], torch.Tensor] | None = None,
) -> Iterator[AdjointStepCompleted]:
    """``src/pyshocks/timestepping.py:155-215``: the reverse sweep over the
    checkpoints saved by :func:`step`, with dt re-read from them (frozen).

    For a stepper built by :func:`make_time_stepper` each transpose step is a
    matrix-free CUDA transpose of the whole ghosted step
    (``shk_ssprk33_vjp_ghosted_f64``) instead of a dense ``jax.jacfwd``
    Jacobian, with the reference's semantics: ghost entries of *p* reach the
    interior through the operator's ghost rows, and ghost entries pass through.
    Schemes: Rusanov (any alpha) or global Lax-Friedrichs with the constant or
    WENO-JS5 reconstruction (the reference adjoint driver's ``lf`` scheme with
    the default reconstruction, ``drivers/burgers-adjoint.py:380-408``)."""
    if stepper.checkpoint is None:
        raise ValueError("Adjoint time stepping requires a checkpoint.")
    src = stepper.source
    from pyshocks_gb300 import adjoint as adj
    from pyshocks_gb300 import burgers

    gpu = isinstance(src, OperatorSource) and isinstance(src.scheme, burgers.GpuConservationLawScheme)
    fused = gpu and burgers.ghosted_supported(src.scheme)
    if gpu and not fused:
        raise NotImplementedError("the single-instance adjoint covers Rusanov and Lax-Friedrichs "
                                  "with the constant or WENO-JS5 reconstruction (batched plans: "
                                  "Rusanov with WENO-JS5 or the learned reconstruction)")

    def _vjp(dt, t, u, p):
        if fused:
            return adj.vjp_step(src.scheme, src.grid, dt, u, p, bc=src.bc, t=float(t))
        # generic closures: differentiate advance() with torch (dt, t constant)
        _, fn = torch.func.vjp(lambda v: advance(stepper, dt, t, v), u)
        return fn(p)[0]

    def _load(m):
        # file checkpoints return host arrays: the state goes back to p's device
        chk = dict(load(stepper.checkpoint, m))
        if not isinstance(chk["u"], torch.Tensor):
            chk["u"] = torch.as_tensor(chk["u"], device=p0.device)
        # float64 either way: a stored float, a 0-d array or a 0-d tensor
        chk["t"] = _as_float(chk["t"]) if isinstance(chk["t"], torch.Tensor) else float(chk["t"])
        chk["m"] = int(chk["m"])
        return chk

    chk = _load(maxit)
    assert chk["m"] == maxit
    t = tfinal = chk["t"]
    p = p0
    if apply_boundary is not None:
        p = apply_boundary(chk["t"], chk["u"], p)
    yield AdjointStepCompleted(t=t, tfinal=tfinal, dt=0.0, iteration=maxit, u=chk["u"], p=p)
    for m in range(maxit - 1, -1, -1):
        chk = _load(m)
        dt = t - chk["t"]
        assert chk["m"] == m
        p = _vjp(dt, chk["t"], chk["u"], p)
        if apply_boundary is not None:
            p = apply_boundary(chk["t"], chk["u"], p)
        t = chk["t"]
        yield AdjointStepCompleted(t=t, tfinal=tfinal, dt=dt, iteration=m, u=chk["u"], p=p)
