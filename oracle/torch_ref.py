"""torch-CPU float64 restatement of the same path, for derivatives.

THIS IS TEST INFRASTRUCTURE (the oracle), like ``oracle/numpy_ref.py``: only
tests, ``smoke()`` and the bench's CPU legs use it, never the product.

JAX is not installed, so ``torch.autograd`` stands in for the reference's
``jax.jacfwd`` in ``adjoint_step`` (``src/pyshocks/timestepping.py:155-215``):
the transpose Jacobian-vector product of one SSPRK33 step with the time step
``dt`` frozen (``timestepping.py:200-206``). Conventions at non-differentiable
points are torch's, which coincide with JAX's: ``d|u|/du = 0`` at ``u = 0``
and ``max(a, b)`` splits the cotangent evenly at ties.

Arrays are batched periodic interiors of shape ``(B, N)`` (no ghost cells):
with periodic boundaries and stencil reach 3 the interior of
``apply_operator`` equals circular indexing (``src/pyshocks/scalar.py:529-540``
fills the ghosts with interior copies and zero padding only reaches ghost
outputs).
"""

from __future__ import annotations

import math

import torch

# WENO-JS 5/3 coefficients (src/pyshocks/weno.py:206-244)
_A53 = (13.0 / 12.0, 1.0 / 4.0)
_D53 = (1.0 / 10.0, 6.0 / 10.0, 3.0 / 10.0)


def _sh(u: torch.Tensor, k: int) -> torch.Tensor:
    """``u[i + k]`` with periodic wrap along the last axis."""
    return torch.roll(u, shifts=-k, dims=-1)


def weno53_side(u: torch.Tensor, eps: float) -> torch.Tensor:
    """Value at ``x_{i+1/2}`` reconstructed from cell ``i``
    (``src/pyshocks/reconstruction.py:351-355``, ``weno.py:114-157,247-256``)."""
    um2, um1, u0, up1, up2 = _sh(u, -2), _sh(u, -1), u, _sh(u, 1), _sh(u, 2)
    b0 = _A53[0] * (u0 - 2 * um1 + um2) ** 2 + _A53[1] * (3 * u0 - 4 * um1 + um2) ** 2
    b1 = _A53[0] * (up1 - 2 * u0 + um1) ** 2 + _A53[1] * (up1 - um1) ** 2
    b2 = _A53[0] * (up2 - 2 * up1 + u0) ** 2 + _A53[1] * (up2 - 4 * up1 + 3 * u0) ** 2
    a0 = _D53[0] / (eps + b0) ** 2
    a1 = _D53[1] / (eps + b1) ** 2
    a2 = _D53[2] / (eps + b2) ** 2
    s = a0 + a1 + a2
    h0 = (11.0 * u0 - 7.0 * um1 + 2.0 * um2) / 6.0
    h1 = (2.0 * up1 + 5.0 * u0 - um1) / 6.0
    h2 = (-up2 + 5.0 * up1 + 2.0 * u0) / 6.0
    return (a0 / s) * h0 + (a1 / s) * h1 + (a2 / s) * h2


def weno53(u: torch.Tensor, eps: float) -> tuple[torch.Tensor, torch.Tensor]:
    """``(ul, ur)`` (``src/pyshocks/reconstruction.py:358-377``): ``ul`` is the
    mirrored reconstruction at ``x_{i-1/2}``."""
    ur = weno53_side(u, eps)
    ul = torch.flip(weno53_side(torch.flip(u, dims=(-1,)), eps), dims=(-1,))
    return ul, ur


# WENO-JS 3/2 coefficients (src/pyshocks/weno.py:166-203)
_D32 = (1.0 / 3.0, 2.0 / 3.0)


def weno32_side(u: torch.Tensor, eps: float) -> torch.Tensor:
    """WENO-JS 3/2 value at ``x_{i+1/2}`` from cell ``i`` (``weno.py:166-203``,
    ``:247-256``): beta = ((u_i - u_{i-1})^2, (u_{i+1} - u_i)^2),
    uhat = (3/2 u_i - 1/2 u_{i-1}, 1/2 (u_i + u_{i+1}))."""
    um1, u0, up1 = _sh(u, -1), u, _sh(u, 1)
    a0 = _D32[0] / (eps + (u0 - um1) ** 2) ** 2
    a1 = _D32[1] / (eps + (up1 - u0) ** 2) ** 2
    s = a0 + a1
    return (a0 / s) * (1.5 * u0 - 0.5 * um1) + (a1 / s) * (0.5 * up1 + 0.5 * u0)


def weno32(u: torch.Tensor, eps: float) -> tuple[torch.Tensor, torch.Tensor]:
    """``(ul, ur)`` of WENO-JS 3/2 (``reconstruction.py:358-377``)."""
    ur = weno32_side(u, eps)
    ul = torch.flip(weno32_side(torch.flip(u, dims=(-1,)), eps), dims=(-1,))
    return ul, ur


def _es_weno32_weights(u: torch.Tensor, eps: float) -> tuple[torch.Tensor, torch.Tensor]:
    """ES-WENO weights (``src/pyshocks/weno.py:284-296``) of the right side."""
    um1, u0, up1 = _sh(u, -1), u, _sh(u, 1)
    b0 = (u0 - um1) ** 2
    b1 = (up1 - u0) ** 2
    tau = (up1 - 2 * u0 + um1) ** 2
    a0 = _D32[0] * (1 + tau / (eps + b0))
    a1 = _D32[1] * (1 + tau / (eps + b1))
    s = a0 + a1
    return a0 / s, a1 / s


def esweno32_side(u: torch.Tensor, eps: float) -> torch.Tensor:
    """``src/pyshocks/reconstruction.py:413-417``."""
    um1, u0, up1 = _sh(u, -1), u, _sh(u, 1)
    w0, w1 = _es_weno32_weights(u, eps)
    h0 = 1.5 * u0 - 0.5 * um1
    h1 = 0.5 * up1 + 0.5 * u0
    return w0 * h0 + w1 * h1


def esweno32(u: torch.Tensor, eps: float) -> tuple[torch.Tensor, torch.Tensor]:
    ur = esweno32_side(u, eps)
    ul = torch.flip(esweno32_side(torch.flip(u, dims=(-1,)), eps), dims=(-1,))
    return ul, ur


def physical_flux(equation: str, u: torch.Tensor) -> torch.Tensor:
    if equation == "burgers":
        return u**2 / 2
    if equation == "advection":
        return 1.0 * u
    if equation == "lwr":
        return u * (1 - u)
    raise ValueError(equation)


def wavespeed(equation: str, u: torch.Tensor) -> torch.Tensor:
    if equation == "burgers":
        return u
    if equation == "advection":
        return torch.ones_like(u)
    if equation == "lwr":
        return 1 - 2 * u
    raise ValueError(equation)


def face_flux(
    u: torch.Tensor,
    *,
    flux_kind: str = "rusanov",
    rec: str = "wenojs53",
    eps: float = 1.0e-6,
    delta: float = 1.0e-6,
    equation: str = "burgers",
    weights=None,
) -> torch.Tensor:
    """Numerical flux at face ``i+1/2`` for every cell ``i`` (periodic)."""
    if rec == "wenojs53":
        ul, ur = weno53(u, eps)
    elif rec == "esweno32":
        ul, ur = esweno32(u, eps)
    elif rec == "wenojs32":
        ul, ur = weno32(u, eps)
    elif rec == "constant":
        # reconstruction.py:153-163
        ul, ur = u, u
    elif rec == "learned":
        from oracle.learned_ref import learned_recon

        ul, ur = learned_recon(u, weights, eps)
    else:
        raise ValueError(rec)
    ulp = _sh(ul, 1)  # left value in cell i+1
    up = _sh(u, 1)
    fl = physical_flux(equation, ulp)
    fr = physical_flux(equation, ur)
    if flux_kind in {"rusanov", "lf"}:
        a = torch.abs(wavespeed(equation, u))
        if flux_kind == "lf":
            # src/pyshocks/scalar.py:277 -- global maximum per instance
            amax = torch.amax(a, dim=-1, keepdim=True)
        else:
            # src/pyshocks/scalar.py:243-246 -- cell values, not reconstructed
            amax = torch.maximum(_sh(a, 1), a)
        # src/pyshocks/scalar.py:248
        return 0.5 * (fl + fr) - 0.5 * amax * (ulp - ur)
    if flux_kind == "godunov":
        # src/pyshocks/scalar.py:91-132 with a = u (burgers/schemes.py:83-89):
        # the reconstructed speeds are the reconstructed states
        return torch.where((ur + ulp) / 2 > 0, fr, fl)
    if flux_kind == "eo":
        # src/pyshocks/scalar.py:287-322, omega = 0 (burgers/schemes.py:184-196)
        zero = torch.zeros_like(u)
        return (physical_flux(equation, torch.maximum(ur, zero))
                + physical_flux(equation, torch.minimum(ulp, zero))
                - physical_flux(equation, zero))
    if flux_kind == "esweno":
        # src/pyshocks/scalar.py:91-132 upwind with a = u, then the ES-WENO
        # dissipation of src/pyshocks/burgers/schemes.py:242-256
        aavg = (ur + ulp) / 2
        fnum = torch.where(aavg > 0, fr, fl)
        w0, _ = _es_weno32_weights(u, eps)
        dw = _sh(w0, 1) - w0
        mu = torch.sqrt(dw**2 + delta**2) / 8.0
        gnum = -(mu + dw / 8.0) * (up - u)
        return fnum + gnum
    raise ValueError(flux_kind)


def apply_operator(u: torch.Tensor, dx, **kw) -> torch.Tensor:
    """``-(F_{i+1/2} - F_{i-1/2}) / dx`` (``src/pyshocks/schemes.py:339-346``)."""
    f = face_flux(u, **kw)
    dx = torch.as_tensor(dx, dtype=u.dtype).reshape(-1, 1) if u.dim() > 1 else dx
    return -(f - _sh(f, -1)) / dx


def ssprk33(u: torch.Tensor, dt, dx, **kw) -> torch.Tensor:
    """``src/pyshocks/timestepping.py:312-320``; *dt* is a per-instance column."""
    dt = torch.as_tensor(dt, dtype=u.dtype).reshape(-1, 1) if u.dim() > 1 else dt
    k1 = u + dt * apply_operator(u, dx, **kw)
    k2 = 3.0 / 4.0 * u + 1.0 / 4.0 * (k1 + dt * apply_operator(k1, dx, **kw))
    return 1.0 / 3.0 * u + 2.0 / 3.0 * (k2 + dt * apply_operator(k2, dx, **kw))


def predict_dt(u: torch.Tensor, dx, theta: float = 1.0, equation: str = "burgers"):
    """``theta * 0.5 dx / max|f'(u)|`` + the ``1e-15`` of
    ``src/pyshocks/timestepping.py:139-142`` (no final-time clip)."""
    smax = torch.amax(torch.abs(wavespeed(equation, u)), dim=-1)
    dx = torch.as_tensor(dx, dtype=u.dtype)
    return theta * (0.5 * dx / smax) + 1.0e-15


def forward(u0: torch.Tensor, dx, nsteps: int, theta: float = 1.0, dts=None, **kw):
    """Run *nsteps* SSPRK33 steps. With ``dts=None`` the per-instance time steps
    are predicted (and detached, as the reference freezes them); otherwise the
    given ``(nsteps, B)`` sequence is used. Returns ``(u, dts)``."""
    u = u0
    out_dts = []
    equation = kw.get("equation", "burgers")
    for m in range(nsteps):
        if dts is None:
            with torch.no_grad():
                dt = predict_dt(u.detach(), dx, theta, equation)
        else:
            dt = dts[m]
        out_dts.append(dt)
        u = ssprk33(u, dt, dx, **kw)
    return u, torch.stack(out_dts) if out_dts else None


def adjoint_gradient(u0, u_target, dx, nsteps, theta=1.0, dts=None, **kw):
    """``dJ/du0`` for ``J = 0.5 * sum (u(T) - u_target)^2`` with frozen ``dt``."""
    u0 = u0.detach().clone().requires_grad_(True)
    if dts is None:
        _, dts = forward(u0.detach(), dx, nsteps, theta, **kw)
    uT, _ = forward(u0, dx, nsteps, theta, dts=dts, **kw)
    J = 0.5 * torch.sum((uT - u_target) ** 2)
    (g,) = torch.autograd.grad(J, u0)
    return g, J.detach(), dts


def step_vjp(u: torch.Tensor, p: torch.Tensor, dt, dx, **kw) -> torch.Tensor:
    """``(d step / d u)^T p`` of one SSPRK33 step at state *u*, *dt* frozen
    (``src/pyshocks/timestepping.py:205-206``)."""
    u = u.detach().clone().requires_grad_(True)
    out = ssprk33(u, dt, dx, **kw)
    (g,) = torch.autograd.grad(out, u, grad_outputs=p)
    return g


def exact_cell_average_sine_periodic(n: int, a: float = -1.0, b: float = 1.0, mean=0.5):
    h = (b - a) / n
    f = torch.linspace(a, b, n + 1, dtype=torch.float64)
    return mean + (torch.cos(math.pi * f[:-1]) - torch.cos(math.pi * f[1:])) / (math.pi * h)


# {{{ one ghosted instance: the reference's array arithmetic (adjoint_step)

# The single-instance adjoint_step of the reference (src/pyshocks/timestepping.py:
# 155-215) differentiates advance() over the whole ghosted array of n + 2g
# cells. These functions restate that array arithmetic in torch, so that
# torch.func.vjp gives the same J^T p as jax.jacfwd (both exact derivatives;
# max() and |.| share JAX's conventions: an even split at ties, d|x|/dx(0) = 0):
#   ghost fill        src/pyshocks/scalar.py:419-429 (Dirichlet), 469-495
#                     (Neumann), 529-540 (periodic: right ghosts, then left)
#   reconstruction    src/pyshocks/reconstruction.py:153-163 (constant),
#                     351-377 (WENO-JS5, zero-padded "same" convolutions,
#                     src/pyshocks/convolve.py:113-114)
#   Rusanov / LF      src/pyshocks/scalar.py:192-278 (zero-padded face array)
#   operator, SSPRK33 src/pyshocks/schemes.py:339-346, timestepping.py:312-320
# They are pinned to the NumPy oracle (oracle/numpy_ref.py, itself pinned to
# the reference's own runs, ghost entries included) by tests/test_oracle.py.


def _conv_same(u: torch.Tensor, taps) -> torch.Tensor:
    """``numpy.convolve(u, taps, mode="same")`` (zero padding) of a 1D tensor,
    taps ordered ``(i + h, ..., i - h)``."""
    k = len(taps)
    h = k // 2
    m = u.shape[-1]
    up = torch.nn.functional.pad(u, (h, h))
    return sum(float(taps[j]) * up[2 * h - j: 2 * h - j + m] for j in range(k) if taps[j] != 0.0)


def _weno53_side_ghosted(f: torch.Tensor, eps: float) -> torch.Tensor:
    from oracle.numpy_ref import weno_js_53_coefficients

    s = weno_js_53_coefficients()
    beta = [sum(float(s.a[j]) * _conv_same(f, s.b[i, j]) ** 2 for j in range(s.a.size))
            for i in range(3)]
    uhat = [_conv_same(f, s.c[i]) for i in range(3)]
    alpha = [float(s.d[i, 0]) / (eps + beta[i]) ** 2 for i in range(3)]
    tot = alpha[0] + alpha[1] + alpha[2]
    return sum((alpha[i] / tot) * uhat[i] for i in range(3))


def ghosted_fill(u: torch.Tensor, g: int, bc: dict, stage: int, x: torch.Tensor) -> torch.Tensor:
    """The boundary's ghost overwrite of a ghosted array (out of place).
    ``bc``: ``{"left": kind, "right": kind, "dirichlet": [stage][side][k],
    "neumann": [stage][side]}``, kind in periodic / dirichlet / neumann; *x*:
    the cell centres (the Neumann mirror distance, scalar.py:494)."""
    m = u.shape[0]
    n = m - 2 * g
    if bc["left"] == "periodic":
        return torch.cat([u[n:n + g], u[g:g + n], u[g:2 * g]])
    parts = []
    for side in (0, 1):
        kind = bc["left"] if side == 0 else bc["right"]
        # ghost cells ordered along the array; k = distance from the interior
        ks = range(g - 1, -1, -1) if side == 0 else range(g)
        vals = []
        for k in ks:
            ito = g - 1 - k if side == 0 else g + n + k
            if kind == "dirichlet":
                vals.append(torch.tensor(float(bc["dirichlet"][stage][side][k]), dtype=u.dtype))
            else:
                ifrom = g + k if side == 0 else g + n - 1 - k
                sgn = -1.0 if side == 0 else 1.0
                vals.append(u[ifrom] + sgn * float(x[ifrom] - x[ito]) * float(bc["neumann"][stage][side]))
        parts.append(torch.stack(vals) if vals else u[:0])
    return torch.cat([parts[0], u[g:g + n], parts[1]])


def ghosted_operator(u: torch.Tensor, dx: float, g: int, bc: dict, stage: int, x: torch.Tensor, *,
                     rec: str = "wenojs53", flux_kind: str = "rusanov", eps: float = 1.0e-6,
                     nu: float = 1.0, equation: str = "burgers") -> torch.Tensor:
    """``apply_operator`` on every cell of the ghosted array (ghosts included)."""
    v = ghosted_fill(u, g, bc, stage, x)
    if rec == "constant":
        ul = ur = v
    else:
        ur = _weno53_side_ghosted(v, eps)
        ul = torch.flip(_weno53_side_ghosted(torch.flip(v, (0,)), eps), (0,))
    fl = physical_flux(equation, ul)
    fr = physical_flux(equation, ur)
    a = torch.abs(wavespeed(equation, v))
    a = torch.amax(a) if flux_kind == "lf" else torch.maximum(a[1:], a[:-1])
    fnum = 0.5 * (fl[1:] + fr[:-1]) - 0.5 * a * nu * (ul[1:] - ur[:-1])
    f = torch.nn.functional.pad(fnum, (1, 1))
    return -(f[1:] - f[:-1]) / dx


def ghosted_advance(u: torch.Tensor, dt: float, dx: float, g: int, bc: dict, x: torch.Tensor,
                    **kw) -> torch.Tensor:
    """SSPRK33 ``advance`` on the raw ghosted array, the boundary at each stage."""
    k1 = u + dt * ghosted_operator(u, dx, g, bc, 0, x, **kw)
    k2 = 3.0 / 4.0 * u + 1.0 / 4.0 * (k1 + dt * ghosted_operator(k1, dx, g, bc, 1, x, **kw))
    return 1.0 / 3.0 * u + 2.0 / 3.0 * (k2 + dt * ghosted_operator(k2, dx, g, bc, 2, x, **kw))


def ghosted_step_vjp(u: torch.Tensor, p: torch.Tensor, dt: float, dx: float, g: int, bc: dict,
                     x: torch.Tensor, **kw) -> torch.Tensor:
    """``jac.T @ p`` of one ghosted step (timestepping.py:174, 205-206)."""
    _, fn = torch.func.vjp(lambda v: ghosted_advance(v, dt, dx, g, bc, x, **kw), u)
    return fn(p)[0]


# }}}
