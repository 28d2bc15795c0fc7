"""Batched inverse problems: recover initial states from final observations.

Each iteration of the gradient descent is one forward solve with sqrt(n)
checkpoints, the misfit ``J_b = 1/2 sum_i (u_b(T)_i - obs_b,i)^2`` reduced in
float64 per instance, one reverse sweep of the hand-written adjoint (dt frozen,
as ``adjoint_step`` in ``src/pyshocks/timestepping.py:155-215``) and a
projected update ``u0 <- clip(u0 - lr * g, lo, hi)``. None of these allocate or
synchronise, so a whole iteration is captured once in a CUDA graph and
replayed.
"""

from __future__ import annotations

import numpy as np
import torch

from pyshocks_gb300.adjoint import CheckpointedSolve
from pyshocks_gb300.batched import BatchedSolver


class InverseProblem:
    """Gradient-descent recovery of the initial states of a batch.

    :arg scheme: a scheme of :mod:`pyshocks_gb300.burgers` (e.g. ``LWRRusanov``
        with a :class:`~pyshocks_gb300.learned.LearnedWENO` reconstruction).
    :arg sizes: cells of every instance; ``dx`` their cell sizes.
    :arg nsteps: SSPRK33 steps of every forward solve.
    :arg bounds: box constraint of the projected update (``(0, 1)`` for
        densities).
    :arg lr: gradient step (the misfit is an unweighted sum over cells).
    """

    def __init__(self, scheme, sizes, dx, nsteps: int, *, dtype=torch.float32,
                 theta: float = 1.0, stride: int | None = None, bounds=(0.0, 1.0),
                 lr: float = 1.0):
        self.solver = BatchedSolver(scheme, sizes, dx, theta=theta, dtype=dtype, max_steps=nsteps)
        self.cs = CheckpointedSolve(self.solver, nsteps, stride)
        dev = self.solver.device
        self.inst = torch.repeat_interleave(torch.arange(self.solver.B, device=dev),
                                            torch.tensor(self.solver.sizes, device=dev))
        self.u0 = torch.zeros(self.solver.total, dtype=dtype, device=dev)
        self.obs = torch.zeros_like(self.u0)
        self.J = torch.zeros(self.solver.B, dtype=torch.float64, device=dev)
        self.bounds = bounds
        # J is a plain sum over cells and the solution operator is close to a
        # transport (norm-preserving away from shocks), so dJ/du0 is O(residual)
        # and a step of lr ~ 1 is the natural scale
        self.lr = float(lr)
        self.graph = None

    def forward(self, u0: torch.Tensor) -> torch.Tensor:
        return self.cs.forward(u0)

    def observe(self, u_true: torch.Tensor) -> None:
        """Observations = the final state of a forward solve from *u_true*."""
        self.obs.copy_(self.forward(u_true.reshape(-1).to(self.u0)))

    def _iteration(self) -> None:
        uT = self.cs.forward(self.u0)
        r = uT - self.obs
        self.J.zero_()
        self.J.index_add_(0, self.inst, 0.5 * r.double() ** 2)
        g = self.cs.backward(r)
        self.u0.sub_(self.lr * g).clamp_(*self.bounds)

    def run(self, u_init: torch.Tensor, iters: int, *, graph: bool = True) -> list[torch.Tensor]:
        """*iters* gradient steps from *u_init*; returns the misfit per
        iteration (one ``J[B]`` tensor each, misfit of the iterate before the
        step)."""
        self.u0.copy_(u_init.reshape(-1).to(self.u0))
        hist = []
        if not graph:
            for _ in range(iters):
                self._iteration()
                hist.append(self.J.clone())
            return hist
        if self.graph is None:
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):  # warm-up outside the capture
                saved = self.u0.clone()
                self._iteration()
                self.u0.copy_(saved)
            torch.cuda.current_stream().wait_stream(side)
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph):
                self._iteration()
            self.u0.copy_(u_init.reshape(-1).to(self.u0))
        for _ in range(iters):
            self.graph.replay()
            hist.append(self.J.clone())
        return hist


def lwr_initial_states(rng: np.random.Generator, sizes, device="cuda", plateau: float = 0.95):
    """Exact cell averages of ``clip(0.5 + 0.3 sum_k A_k sin(k pi x + phi_k), 0, 1)``
    (8 modes, A_k ~ N(0, 1)/k^2) with 2 jam plateaus at ``plateau`` (centre
    U(-1, 1), width U(0.05, 0.2), periodic), packed."""
    rows = []
    for n in sizes:
        f = torch.linspace(-1.0, 1.0, int(n) + 1, dtype=torch.float64, device=device)
        fl, fr = f[:-1], f[1:]
        h = fr - fl
        base = torch.zeros_like(fl)
        for k in range(1, 9):
            a = rng.normal() / k**2
            ph = rng.uniform(0, 2 * np.pi)
            base += a * (torch.cos(k * np.pi * fl + ph) - torch.cos(k * np.pi * fr + ph)) / (k * np.pi * h)
        rho = 0.5 + 0.3 * base
        for _ in range(2):
            c, w = rng.uniform(-1, 1), rng.uniform(0.05, 0.2)
            frac = torch.zeros_like(rho)
            for sh in (-2.0, 0.0, 2.0):
                lo, hi = c - w / 2 + sh, c + w / 2 + sh
                frac += torch.clamp((torch.minimum(fr, torch.full_like(fr, hi))
                                     - torch.maximum(fl, torch.full_like(fl, lo))) / h, 0.0, 1.0)
            frac = torch.clamp(frac, max=1.0)
            rho = (1 - frac) * rho + frac * plateau
        rows.append(torch.clamp(rho, 0.0, 1.0))
    return torch.cat(rows)
