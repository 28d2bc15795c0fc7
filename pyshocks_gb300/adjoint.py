"""Discrete adjoint of the batched SSPRK33 / WENO-JS5 / Rusanov solve.

The reference differentiates one step with ``jax.jacfwd(advance)`` and applies
``p <- jac.T @ p`` backwards over checkpoints saved at *every* step, with the
time step re-read from the checkpoints rather than differentiated
(``src/pyshocks/timestepping.py:155-215``). Here:

* the transpose Jacobian-vector product of a step is a matrix-free CUDA kernel
  (``shk_plan_adjoint``): no dense ``(N+6)^2`` Jacobian;
* states are checkpointed every ``stride ~ sqrt(nsteps)`` steps on the device and
  each segment is recomputed with the recorded dt before it is swept
  backwards;
* dt is frozen exactly as in the reference.

Cotangents are defined on the interior cells (the packed layout). With the
reference's ghosted layout, a cotangent with zero ghost entries maps to the
same interior result, because interior outputs do not depend on input ghosts
(the boundary fill overwrites them).
"""

from __future__ import annotations

import ctypes

import math

import torch

from pyshocks_gb300 import _lib as L
from pyshocks_gb300.batched import BatchedSolver


class CheckpointedSolve:
    """Forward run with sqrt(n) checkpoints and its reverse sweep.

    :arg solver: a :class:`BatchedSolver` created with ``max_steps >= nsteps``.
    :arg nsteps: number of SSPRK33 steps of the forward run.
    :arg stride: checkpoint interval (default ``ceil(sqrt(nsteps))``).
    :arg store_stages: keep what each replayed step's reverse step would
        recompute (its stage states, and for double WENO-JS5 on periodic
        instances the face values of u, k1 and k2: ``stride x`` 2 float or 8
        double arrays of the batch) so that the reverse steps skip their
        forward stages (same result, bit for bit). Left out when it would take
        more than half of the free device memory.
    """

    def __init__(self, solver: BatchedSolver, nsteps: int, stride: int | None = None,
                 store_stages: bool = True):
        if solver.max_steps < nsteps:
            raise ValueError("the solver's dt history must hold every step (max_steps >= nsteps)")
        self.solver = solver
        self.nsteps = int(nsteps)
        self.stride = int(stride or max(1, math.ceil(math.sqrt(max(1, nsteps)))))
        nck = max(1, -(-self.nsteps // self.stride))
        dev, dt = solver.device, solver.dtype
        self.ckpt = torch.empty((nck, solver.total), dtype=dt, device=dev)
        self.seg = torch.empty((self.stride, solver.total), dtype=dt, device=dev)
        self.p_a = torch.empty(solver.total, dtype=dt, device=dev)
        self.p_b = torch.empty(solver.total, dtype=dt, device=dev)
        nb = ctypes.c_int64(0)
        L.check(solver.lib.shk_plan_adjoint_stage_bytes(solver._plan, ctypes.byref(nb)),
                "plan_adjoint_stage_bytes")
        want = store_stages and nb.value > 0
        if want:
            # stage storage is an optimisation: leave it out when it would take
            # more than half of the free device memory
            free, _ = torch.cuda.mem_get_info(dev)
            want = self.stride * nb.value <= free // 2
        self.stages = (torch.empty((self.stride, nb.value), dtype=torch.uint8, device=dev)
                       if want else None)

    def forward(self, u0: torch.Tensor, *, t0=None, tfinal=None) -> torch.Tensor:
        """Run the forward solve from *u0*; returns the final packed state."""
        s = self.solver
        s.reset(u0, t0=t0, tfinal=tfinal)
        L.check(
            s.lib.shk_plan_forward_checkpointed(
                s._plan, s.buf_a.data_ptr(), s.buf_b.data_ptr(), self.nsteps,
                self.ckpt.data_ptr(), self.stride, L.stream_handle()),
            "plan_forward_checkpointed",
        )
        s._steps += self.nsteps
        return s.u

    def backward(self, p_final: torch.Tensor) -> torch.Tensor:
        """``dJ/du0`` given ``dJ/du(T)`` (packed); dt frozen."""
        s = self.solver
        self.p_a.copy_(p_final.reshape(-1).to(self.p_a))
        L.check(
            s.lib.shk_plan_adjoint_staged(
                s._plan, self.ckpt.data_ptr(), self.stride, self.nsteps, self.seg.data_ptr(),
                L.ptr(self.stages), self.p_a.data_ptr(), self.p_b.data_ptr(),
                L.stream_handle()),
            "plan_adjoint",
        )
        return (self.p_a if self.nsteps % 2 == 0 else self.p_b).clone()


class _SolveFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, solve, t0, tfinal):
        ctx.solve = solve
        return solve.forward(u0.detach(), t0=t0, tfinal=tfinal).clone()

    @staticmethod
    def backward(ctx, grad):
        return ctx.solve.backward(grad.contiguous()), None, None, None


def solve(u0: torch.Tensor, checkpointed: CheckpointedSolve, *, t0=None, tfinal=None):
    """Differentiable batched solve: ``u(T) = solve(u0)``; ``backward`` runs the
    hand-written adjoint with the dt sequence of the forward run frozen."""
    return _SolveFn.apply(u0, checkpointed, t0, tfinal)


def vjp_step(scheme, grid, dt: float, u: torch.Tensor, p_next: torch.Tensor, *,
             bc=None, t: float = 0.0) -> torch.Tensor:
    """``(d advance / d u)^T p_next`` of one SSPRK33 step of a ghosted single
    instance: the ``jac.T @ p`` of ``src/pyshocks/timestepping.py:174,205-206``
    with ``jac`` the Jacobian of the whole ghosted step (``shk_ssprk33_vjp_ghosted_f64``):
    ghost entries of *p_next* reach the interior through the operator's ghost
    rows, as they do in the reference. With a Dirichlet / Neumann *bc* the step
    from time *t* is transposed exactly, the boundary data entering as
    constants. Rusanov (any alpha) or global Lax-Friedrichs with the constant
    or WENO-JS5 reconstruction."""
    for name, arr in (("u", u), ("p", p_next)):
        if not (arr.is_cuda and arr.dtype == torch.float64 and arr.is_contiguous()
                and arr.shape[0] == grid.x.shape[0]):
            raise ValueError(f"{name}: expected a contiguous float64 CUDA array of {grid.x.shape[0]}")
    from pyshocks_gb300.burgers import c_boundary, ghosted_workspace

    out = torch.empty_like(u)
    cb = None
    if bc is not None:
        dt_ = float(dt)
        cb = c_boundary(bc, grid, (float(t), float(t) + dt_, float(t) + 0.5 * dt_))
    ws = ghosted_workspace(grid, u.device)
    L.check(
        L.lib().shk_ssprk33_vjp_ghosted_f64(scheme.c_scheme(grid.dx_min),
                                            None if cb is None else ctypes.byref(cb), u.data_ptr(),
                                            p_next.data_ptr(), out.data_ptr(), grid.ncells,
                                            grid.nghosts, float(grid.dx_min), float(dt),
                                            ws.data_ptr(), ws.numel(), L.stream_handle()),
        "ssprk33_vjp_ghosted",
    )
    return out
