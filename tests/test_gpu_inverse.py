"""Batched LWR inverse problem (learned-weight scheme, float32 state, float64
misfits): gradient descent with the hand-written adjoint (MLP backward
included), with and without the whole iteration captured in a CUDA graph."""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _problem(graph_sizes=(256, 512, 384, 256), nsteps=60):
    from pyshocks_gb300 import burgers, learned
    from pyshocks_gb300.inverse import InverseProblem

    rec = learned.LearnedWENO(params=learned.init_params(seed=2))
    scheme = burgers.LWRRusanov(rec=rec)
    sizes = list(graph_sizes)
    return InverseProblem(scheme, sizes, [2.0 / n for n in sizes], nsteps, lr=0.5), sizes


def test_gradient_descent_reduces_misfit_and_graph_matches_eager():
    from pyshocks_gb300.inverse import lwr_initial_states

    rng = np.random.default_rng(5)
    prob, sizes = _problem()
    truth = lwr_initial_states(rng, sizes)
    prob.observe(truth)
    # initial guess: the instance means (the conserved mass is known)
    guess = torch.cat([torch.full((n,), float(x.mean()), dtype=torch.float64, device="cuda")
                       for n, x in zip(sizes, torch.split(truth, sizes))])
    eager = prob.run(guess, 8, graph=False)
    j_eager = torch.stack(eager).cpu().numpy()
    prob2, _ = _problem()
    prob2.observe(truth)
    graphed = prob2.run(guess, 8, graph=True)
    j_graph = torch.stack(graphed).cpu().numpy()
    assert np.all(np.isfinite(j_graph))
    np.testing.assert_allclose(j_graph, j_eager, rtol=1e-9, atol=0)
    # descent on every instance
    assert np.all(j_eager[-1] < 0.7 * j_eager[0]), (j_eager[0], j_eager[-1])
    assert prob.solver.status() == 0


def test_adjoint_gradient_of_misfit_matches_finite_differences():
    """dJ/du0 . v of a WENO-JS5 LWR solve (float64, smooth initial density)
    against central differences of J, with the recorded dt sequence replayed
    through a fixed-dt table (the adjoint differentiates with dt frozen). The learned reconstruction is not
    used here: its tensor-core inference rounds the network inputs to
    bfloat16, so J has rounding steps that a difference quotient resolves; its
    VJP is checked against autograd of the oracle instead."""
    from pyshocks_gb300 import burgers, reconstruction
    from pyshocks_gb300.adjoint import CheckpointedSolve
    from pyshocks_gb300.batched import BatchedSolver
    from pyshocks_gb300.inverse import lwr_initial_states

    n, nsteps = 256, 30
    rng = np.random.default_rng(9)
    # smooth, unclipped densities: the jam plateaus of lwr_initial_states hold
    # exact ties of the Rusanov max(|f'(L)|, |f'(R)|), where the adjoint takes
    # the even-split subgradient and a one-sided difference quotient does not
    x = torch.linspace(-1.0, 1.0, n + 1, dtype=torch.float64, device="cuda")[:-1] + 1.0 / n
    rho0 = 0.45 + 0.2 * torch.sin(np.pi * x) + 0.05 * torch.cos(3 * np.pi * x + 1.0)
    obs = lwr_initial_states(rng, [n])
    rec = reconstruction.WENOJS53()
    solver = BatchedSolver(burgers.LWRRusanov(rec=rec), [n], 2.0 / n, dtype=torch.float64,
                           max_steps=nsteps)
    cs = CheckpointedSolve(solver, nsteps)
    uT = cs.forward(rho0).clone()  # a view of the solver's buffers, which the reverse sweep reuses
    g = cs.backward(uT - obs)
    dts = solver.dt_history().clone()

    # J with the dt sequence frozen: replay the recorded steps (as the adjoint,
    # which differentiates with dt held fixed)
    def J(u0):
        s2 = BatchedSolver(burgers.LWRRusanov(rec=rec), [n], 2.0 / n, dtype=torch.float64,
                           max_steps=nsteps)
        s2.set_fixed_dt(dts)
        uT2 = CheckpointedSolve(s2, nsteps).forward(u0)
        assert torch.equal(s2.dt_history(), dts)
        return 0.5 * float(torch.sum((uT2 - obs) ** 2))

    # the replay of the unperturbed state is the recorded solve, bit for bit
    assert 0.5 * float(torch.sum((uT - obs) ** 2)) == J(rho0)
    v = torch.tensor(rng.standard_normal(n), device="cuda")
    h = 1.0e-6
    fd = (J(rho0 + h * v) - J(rho0 - h * v)) / (2 * h)
    ad = float(torch.dot(g, v))
    assert abs(fd - ad) < 1.0e-5 * max(1.0, abs(ad)), (fd, ad)


def test_fixed_dt_table_replays_cfl_run_and_scalar_step_matches_maxit():
    from pyshocks_gb300 import burgers, reconstruction
    from pyshocks_gb300.batched import BatchedSolver
    from pyshocks_gb300.timestepping import predict_timestep_from_maxit

    sizes = [200, 320]
    rng = np.random.default_rng(3)
    u0 = torch.tensor(rng.uniform(-1, 1, sum(sizes)), device="cuda")
    a = BatchedSolver(burgers.Rusanov(rec=reconstruction.WENOJS53()), sizes, [2.0 / n for n in sizes], max_steps=40)
    a.reset(u0, tfinal=[0.3, 0.25])
    a.step(40)
    b = BatchedSolver(burgers.Rusanov(rec=reconstruction.WENOJS53()), sizes, [2.0 / n for n in sizes], max_steps=40)
    b.set_fixed_dt(a.dt_history())
    b.reset(u0)
    b.step(41, graph=True)  # the extra step is past the table: a copy-through
    torch.testing.assert_close(b.u, a.u, rtol=0, atol=0)
    torch.testing.assert_close(b.time(), a.time(), rtol=0, atol=0)
    # scalar step: maxit steps of tfinal / maxit + 1e-15 reach tfinal
    maxit, dt = predict_timestep_from_maxit(0.2, 25)
    b.set_fixed_dt(dt, nsteps=maxit)
    b.reset(u0)
    b.step(maxit + 3)
    t = b.time().cpu().numpy()
    np.testing.assert_allclose(t, maxit * dt, rtol=1e-14)
    b.set_fixed_dt(None)
    b.reset(u0, tfinal=0.2)
    b.step(4)
    assert b.status() == 0
