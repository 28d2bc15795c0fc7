"""Discrete adjoint kernels against the torch-CPU float64 autograd oracle (the
stand-in for ``jax.jacfwd`` in ``src/pyshocks/timestepping.py:174``) and
central finite differences with the dt sequence frozen.

Tolerances: one-step VJPs within 1e-11 of autograd relative to the cotangent
scale; multi-step gradients within 1e-9 relative; finite differences
(h = 1e-6) within 1e-5 relative.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import numpy_ref as R
from oracle import torch_ref as T

pytestmark = pytest.mark.gpu


def _scheme(eq="burgers"):
    from pyshocks_gb300 import burgers, reconstruction

    rec = reconstruction.make_reconstruction_from_name("wenojs53", eps=1.0e-6)
    return {"burgers": burgers.Rusanov(rec=rec), "lwr": burgers.LWRRusanov(rec=rec),
            "advection": burgers.AdvectionRusanov(rec=rec)}[eq]


def _interior_vjp(scheme, grid, dt, u, p):
    """``shk_ssprk33_vjp_f64``: the transpose of one step with cotangents on
    the interior cells only (the packed-layout convention of the batched
    adjoint); ghost entries of p are ignored and those of the result are 0."""
    from pyshocks_gb300 import _lib as L

    out = torch.empty_like(u)
    L.check(L.lib().shk_ssprk33_vjp_f64(scheme.c_scheme(grid.dx_min), u.data_ptr(), p.data_ptr(),
                                        out.data_ptr(), grid.ncells, grid.nghosts,
                                        float(grid.dx_min), float(dt), L.stream_handle()))
    return out


def _state(n, seed, eq):
    og = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
    rng = np.random.default_rng(seed)
    return R.lwr_ic(rng, og.f) if eq == "lwr" else R.random_fourier_ic(rng, og.f)


@pytest.mark.parametrize(("n", "eq"), [(64, "burgers"), (300, "burgers"), (1024, "burgers"),
                                        (3001, "burgers"), (512, "lwr"), (256, "advection")])
def test_single_step_vjp_matches_autograd(n, eq):
    import pyshocks_gb300 as gb

    u0 = _state(n, n, eq)
    rng = np.random.default_rng(n + 1)
    p = rng.standard_normal(n + 6)
    dx = 2.0 / n
    ut = torch.tensor(u0[3:-3])[None]
    dt = 0.8 * float(T.predict_dt(ut, dx, equation=eq)[0])
    ref = T.step_vjp(ut, torch.tensor(p[3:-3])[None], dt, dx, equation=eq)[0].numpy()

    grid = gb.make_uniform_cell_grid(-1.0, 1.0, n, nghosts=3)
    out = _interior_vjp(_scheme(eq), grid, dt, torch.tensor(u0, device="cuda"),
                        torch.tensor(p, device="cuda")).cpu().numpy()
    err = np.max(np.abs(out[3:-3] - ref)) / np.max(np.abs(ref))
    assert err < 1.0e-11, err
    np.testing.assert_array_equal(out[:3], 0.0)
    np.testing.assert_array_equal(out[-3:], 0.0)


def test_vjp_at_ties_splits_the_max_evenly():
    """Constant plateaus make |u_i| = |u_{i+1}|: max() ties, where the cotangent
    is split evenly (JAX/torch convention). Inside a plateau L(u) = 0 exactly,
    so the ties survive exactly into k1 and k2 on both sides of the comparison
    (ties created only in exact arithmetic, e.g. a symmetric +a/-a jump, break
    differently under different roundings and are not a meaningful check)."""
    import pyshocks_gb300 as gb

    n = 128
    u = np.full(n, 0.3)
    u[20:70] = 0.95
    u[90:100] = -0.5
    ug = np.concatenate([u[-3:], u, u[:3]])
    p = np.random.default_rng(2).standard_normal(n + 6)
    dx = 2.0 / n
    dt = 0.5 * dx / 0.95
    ref = T.step_vjp(torch.tensor(u)[None], torch.tensor(p[3:-3])[None], dt, dx)[0].numpy()
    grid = gb.make_uniform_cell_grid(-1.0, 1.0, n, nghosts=3)
    out = _interior_vjp(_scheme(), grid, dt, torch.tensor(ug, device="cuda"),
                        torch.tensor(p, device="cuda")).cpu().numpy()[3:-3]
    assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < 1.0e-11


def test_adjoint_step_generator_matches_autograd():
    """The reference-style ``step`` + ``adjoint_step`` pair (InMemoryCheckpoint,
    dt = t_{m+1} - t_m re-read from checkpoints) against autograd through the
    same frozen dt sequence."""
    import pyshocks_gb300 as gb
    from pyshocks_gb300.checkpointing import InMemoryCheckpoint

    n, maxit = 128, 30
    g = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
    u0 = R.exact_cell_average_sine(g)
    grid = gb.make_uniform_cell_grid(-1.0, 1.0, n, nghosts=3)
    bc = gb.scalar.PeriodicBoundary()
    stepper = gb.timestepping.make_time_stepper(_scheme(), grid, bc, theta=1.0,
                                                checkpoint=InMemoryCheckpoint("Iteration"))
    ev = None
    for ev in gb.timestepping.step(stepper, torch.tensor(u0, device="cuda"), maxit=maxit):
        pass
    uT = ev.u
    p0 = uT.clone()  # J = 1/2 |u(T)|^2 over the interior: no ghost cotangent
    p0[:3] = 0.0
    p0[-3:] = 0.0
    dts = []
    for ev in gb.timestepping.adjoint_step(stepper, p0, maxit=maxit):
        if ev.iteration < maxit:
            dts.append(ev.dt)
    grad = ev.p.cpu().numpy()[3:-3]
    dts = torch.tensor(dts[::-1]).reshape(-1, 1)
    u0t = torch.tensor(u0[3:-3])[None]
    ref, _, _ = T.adjoint_gradient(u0t, torch.zeros_like(u0t), 2.0 / n, maxit, dts=dts)
    ref = ref[0].numpy()
    assert np.max(np.abs(grad - ref)) / np.max(np.abs(ref)) < 1.0e-9


@pytest.mark.parametrize("stride", [None, 1, 7])
def test_batched_checkpointed_gradient_matches_autograd(stride):
    """Uneven batch, sqrt(n) checkpoints (and the extremes stride 1, 7),
    J = 1/2 sum (u(T) - u_target)^2 per instance."""
    from pyshocks_gb300.adjoint import CheckpointedSolve
    from pyshocks_gb300.batched import BatchedSolver

    sizes = [64, 50, 1024, 333]
    nsteps = 23
    rng = np.random.default_rng(4)
    u0 = [R.random_fourier_ic(rng, np.linspace(-1, 1, n + 1)) for n in sizes]
    tgt = [R.random_fourier_ic(rng, np.linspace(-1, 1, n + 1)) for n in sizes]
    solver = BatchedSolver(_scheme(), sizes, [2.0 / n for n in sizes], theta=0.9, max_steps=nsteps)
    cs = CheckpointedSolve(solver, nsteps, stride=stride)
    uT = cs.forward(torch.tensor(np.concatenate(u0)))
    tg = torch.tensor(np.concatenate(tgt), device="cuda")
    grad = cs.backward(uT - tg).cpu().numpy()
    hist = solver.dt_history().cpu()
    for b, n in enumerate(sizes):
        ref, _, _ = T.adjoint_gradient(torch.tensor(u0[b])[None], torch.tensor(tgt[b])[None],
                                       2.0 / n, nsteps, dts=hist[:, b].reshape(-1, 1))
        ref = ref[0].numpy()
        got = grad[int(solver.offsets[b]):int(solver.offsets[b + 1])]
        assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1.0e-9, b


def test_gradient_against_central_differences():
    """dJ/du0 . v against (J(u0 + h v) - J(u0 - h v)) / 2h, h = 1e-6, with the dt
    sequence of the unperturbed run frozen (the reference's convention)."""
    from pyshocks_gb300.adjoint import CheckpointedSolve
    from pyshocks_gb300.batched import BatchedSolver

    n, nsteps, B = 256, 40, 2
    rng = np.random.default_rng(8)
    u0 = np.concatenate([R.exact_cell_average_sine(R.make_uniform_cell_grid(-1, 1, n, 3))[3:-3]
                         for _ in range(B)])
    tgt = u0 + 0.05 * rng.standard_normal(u0.size)
    solver = BatchedSolver(_scheme(), [n] * B, 2.0 / n, max_steps=nsteps)
    cs = CheckpointedSolve(solver, nsteps)
    uT = cs.forward(torch.tensor(u0))
    tg = torch.tensor(tgt, device="cuda")
    grad = cs.backward(uT - tg).cpu().numpy()
    dts = solver.dt_history().cpu()
    h = 1.0e-6
    for k in range(4):
        v = rng.standard_normal(u0.size)
        js = []
        for sgn in (+1, -1):
            up = torch.tensor(u0 + sgn * h * v)
            J = 0.0
            for b in range(B):
                sl = slice(b * n, (b + 1) * n)
                out, _ = T.forward(up[sl][None], 2.0 / n, nsteps, dts=dts[:, b].reshape(-1, 1))
                J += 0.5 * float(torch.sum((out[0] - torch.tensor(tgt[sl])) ** 2))
            js.append(J)
        fd = (js[0] - js[1]) / (2 * h)
        ad = float(np.dot(grad, v))
        assert abs(fd - ad) <= 1.0e-5 * max(1.0, abs(ad)), (k, fd, ad)


def test_autograd_function_backward():
    """``adjoint.solve`` inside a torch graph: loss.backward() runs the kernel."""
    from pyshocks_gb300 import adjoint
    from pyshocks_gb300.batched import BatchedSolver

    n, nsteps = 128, 12
    u0 = torch.tensor(R.exact_cell_average_sine(R.make_uniform_cell_grid(-1, 1, n, 3))[3:-3],
                      device="cuda", requires_grad=True)
    solver = BatchedSolver(_scheme(), [n], 2.0 / n, max_steps=nsteps)
    cs = adjoint.CheckpointedSolve(solver, nsteps)
    uT = adjoint.solve(u0, cs)
    loss = 0.5 * torch.sum(uT**2)
    loss.backward()
    ref, _, _ = T.adjoint_gradient(u0.detach().cpu()[None], torch.zeros(1, n, dtype=torch.float64),
                                   2.0 / n, nsteps, dts=solver.dt_history().cpu())
    err = (u0.grad.cpu() - ref[0]).abs().max() / ref.abs().max()
    assert float(err) < 1.0e-9


@pytest.mark.parametrize(("nsteps", "tol"), [(400, 1.0e-5), (4000, 2.0e-5)])
def test_n4096_gradient_16_directions(nsteps, tol):
    """The adjoint benchmark's check at its instance size (N = 4096): dJ/du0
    along 16 random directions against central differences (h = 1e-6) of the
    GPU forward itself, replaying the recorded dt sequence (frozen dt, as
    adjoint_step), with J = 1/2 |u(T) - u_target|^2 and sqrt(n) checkpoints;
    400 steps (before the shock forms) and the configuration's 4000 (t ~ 0.65,
    past it, where a perturbation of h can cross a kink of the Rusanov speed
    max(|u_j|, |u_j+1|) and the central difference sees it; measured worst
    relative mismatch 4e-8 at 400 steps, 3.4e-6 at 4000)."""
    from pyshocks_gb300.adjoint import CheckpointedSolve
    from pyshocks_gb300.batched import BatchedSolver

    n, B = 4096, 2
    rng = np.random.default_rng(31)
    u1 = R.exact_cell_average_sine(R.make_uniform_cell_grid(-1, 1, n, 3))[3:-3]
    u0 = np.tile(u1, B)
    x = np.linspace(-1.0, 1.0, n + 1)[:-1]
    pert = np.concatenate([sum(rng.standard_normal() / k**2 * np.sin(k * np.pi * x + rng.uniform(0, 2 * np.pi))
                               for k in range(1, 9)) for _ in range(B)])
    scheme = _scheme()
    solver = BatchedSolver(scheme, [n] * B, 2.0 / n, max_steps=nsteps)
    cs = CheckpointedSolve(solver, nsteps)
    target = cs.forward(torch.tensor(u0 + 0.05 * pert)).clone()
    uT = cs.forward(torch.tensor(u0))
    grad = cs.backward(uT - target).cpu().numpy()
    replay = BatchedSolver(scheme, [n] * B, 2.0 / n)
    replay.set_fixed_dt(solver.dt_history())

    def J(u):
        replay.reset(torch.tensor(u))
        replay.step(nsteps)
        return 0.5 * float(torch.sum((replay.u - target) ** 2))

    h = 1.0e-6
    worst = 0.0
    for k in range(16):
        v = rng.standard_normal(u0.size)
        fd = (J(u0 + h * v) - J(u0 - h * v)) / (2 * h)
        ad = float(np.dot(grad, v))
        worst = max(worst, abs(fd - ad) / max(1.0, abs(ad)))
        assert abs(fd - ad) <= tol * max(1.0, abs(ad)), (k, fd, ad)
    print(f"N=4096, {nsteps} steps: worst |fd - ad| / max(1, |ad|) over 16 directions {worst:.2e}")


@pytest.mark.parametrize("boundary", ["periodic", "neumann"])
def test_stored_stages_and_faces_give_the_same_gradient(boundary):
    """Plain WENO-JS5 in double: reverse steps that read the replay's stored
    stage states and face values return the recomputing adjoint's gradient bit
    for bit (uneven batch with partial tiles; a boundary plan keeps
    recomputing)."""
    from pyshocks_gb300.adjoint import CheckpointedSolve
    from pyshocks_gb300.batched import BatchedSolver

    sizes = [1024, 700, 2048, 96]
    nsteps = 23
    rng = np.random.default_rng(19)
    u0 = np.concatenate([R.random_fourier_ic(rng, np.linspace(-1, 1, n + 1)) for n in sizes])
    p_T = torch.tensor(rng.standard_normal(u0.size), device="cuda")
    grads = []
    for store in (False, True):
        solver = BatchedSolver(_scheme(), sizes, [2.0 / n for n in sizes], max_steps=nsteps)
        if boundary == "neumann":
            solver.set_boundary("neumann", neumann=[0.0, 0.0])
        cs = CheckpointedSolve(solver, nsteps, stride=5, store_stages=store)
        assert (cs.stages is not None) == (store and boundary == "periodic")
        cs.forward(torch.tensor(u0))
        grads.append(cs.backward(p_T))
        assert solver.status() == 0
    assert torch.equal(grads[0], grads[1])


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_plain_results_do_not_depend_on_the_tile(dtype):
    """Plain WENO-JS5: forward steps and reverse sweeps give the same values,
    bit for bit, at tiles of 64, 512 and 1024 cells (more halo than interior,
    the reverse sweep's default, the float64 forward's default) and in float32
    also 2048 (its forward default; a float64 reverse step of 2048 cells does
    not fit in shared memory). In float32 the forward stage takes two cells
    per lane, so odd instance and stage lengths end a warp's pairs at every
    parity."""
    from pyshocks_gb300.adjoint import CheckpointedSolve
    from pyshocks_gb300.batched import BatchedSolver

    sizes = [4096, 1500, 601, 96, 33]
    nsteps = 9
    rng = np.random.default_rng(47)
    u0 = np.concatenate([R.random_fourier_ic(rng, np.linspace(-1, 1, n + 1)) for n in sizes])
    p_T = torch.tensor(rng.standard_normal(u0.size), device="cuda", dtype=dtype)
    outs, grads = [], []
    for tile in (64, 512, 1024) + ((2048,) if dtype == torch.float32 else ()):
        s = BatchedSolver(_scheme(), sizes, [2.0 / n for n in sizes], tile=tile, max_steps=nsteps,
                          dtype=dtype)
        cs = CheckpointedSolve(s, nsteps, stride=4)
        outs.append(cs.forward(torch.tensor(u0)).clone())
        grads.append(cs.backward(p_T))
        assert s.status() == 0
    for o, g in zip(outs[1:], grads[1:]):
        assert torch.equal(o, outs[0])
        assert torch.equal(g, grads[0])


@pytest.mark.parametrize("boundary", ["periodic", "neumann"])
def test_float32_lwr_steps_do_not_depend_on_the_tile(boundary):
    """The float32 forward step with the LWR flux (the flux sum f(L) + f(R)
    rounded term by term) gives the same states, bit for bit, at every tile,
    periodic or with homogeneous Neumann ghosts."""
    from pyshocks_gb300.batched import BatchedSolver

    sizes = [2048, 1500, 601, 96, 33, 7]
    rng = np.random.default_rng(53)
    u0 = np.concatenate([np.clip(0.5 + 0.3 * R.random_fourier_ic(rng, np.linspace(-1, 1, n + 1)), 0, 1)
                         for n in sizes])
    outs = []
    for tile in (64, 512, 2048):
        s = BatchedSolver(_scheme("lwr"), sizes, [2.0 / n for n in sizes], tile=tile,
                          dtype=torch.float32)
        if boundary == "neumann":
            s.set_boundary("neumann", neumann=(0.0, 0.0))
        s.reset(torch.tensor(u0, dtype=torch.float32))
        outs.append(s.step(40).clone())
        assert s.status() == 0
    assert torch.isfinite(outs[0]).all()
    for o in outs[1:]:
        assert torch.equal(o, outs[0])


def test_step_and_adjoint_step_through_npz_checkpoints(tmp_path):
    """``step`` saving every state to ``.npz`` files (keys m, t, u; the
    reference's ``NumpyCheckpoint``, ``src/pyshocks/checkpointing.py:209-254``)
    and ``adjoint_step`` reading them back give the in-memory run's states and
    gradient bit for bit."""
    import pyshocks_gb300 as gb
    from pyshocks_gb300.checkpointing import InMemoryCheckpoint, NumpyCheckpoint, load

    n, maxit = 96, 12
    g = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
    u0 = torch.tensor(R.exact_cell_average_sine(g), device="cuda")
    grid = gb.make_uniform_cell_grid(-1.0, 1.0, n, nghosts=3)
    bc = gb.scalar.PeriodicBoundary()
    out = {}
    for name, chk in (("mem", InMemoryCheckpoint("Iteration")),
                      ("npz", NumpyCheckpoint("Iteration", dirname=tmp_path))):
        stepper = gb.timestepping.make_time_stepper(_scheme(), grid, bc, theta=1.0,
                                                    checkpoint=chk)
        for ev in gb.timestepping.step(stepper, u0, maxit=maxit):
            pass
        uT = ev.u
        for ev in gb.timestepping.adjoint_step(stepper, uT.clone(), maxit=maxit):
            pass
        out[name] = (uT, ev.p, chk)
    assert torch.equal(out["mem"][0], out["npz"][0])
    assert torch.equal(out["mem"][1], out["npz"][1])
    assert sorted(p.name for p in tmp_path.iterdir())[-1] == f"Iteration_{maxit:09d}.npz"
    last = load(out["npz"][2], maxit)
    assert int(last["m"]) == maxit
    np.testing.assert_array_equal(last["u"], out["mem"][0].cpu().numpy())
