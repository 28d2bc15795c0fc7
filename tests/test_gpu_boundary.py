"""Dirichlet and Neumann boundaries (``src/pyshocks/scalar.py:397-511``) on the
GPU path: the reference's own runs (golden vectors from its source) through
the ``step()`` API, ``apply_operator`` against the oracle at a nonzero time,
and batched plans with time-independent boundary data against the oracle."""

from __future__ import annotations

import pathlib

import numpy as np
import pytest
import torch

from oracle import numpy_ref as R

pytestmark = pytest.mark.gpu

GOLDEN = pathlib.Path(__file__).parent / "golden"


def _golden(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


# the boundary data of the golden runs (tests/golden/make_golden.py)
def dirichlet_torch(t, x):
    return 0.6 + 0.25 * torch.sin(np.pi * x - t)


def dirichlet_np(t, x):
    return 0.6 + 0.25 * np.sin(np.pi * x - t)


def neumann_left(t):
    return 0.3 * np.cos(2.0 * t)


def neumann_right(t):
    return -0.2


def _scheme(flux_kind, rname):
    from pyshocks_gb300 import burgers, reconstruction

    rec = reconstruction.make_reconstruction_from_name(rname, eps=1.0e-6)
    return burgers.make_scheme_from_name(flux_kind, rec=rec)


def _bc(kind):
    from pyshocks_gb300 import scalar

    if kind == "dirichlet":
        return scalar.make_dirichlet_boundary(ga=dirichlet_torch)
    return scalar.make_neumann_boundary(ga=neumann_left, gb=neumann_right)


@pytest.mark.parametrize(("name", "flux_kind", "rname", "kind"), [
    ("dirichlet_rusanov_n128", "rusanov", "wenojs53", "dirichlet"),
    ("neumann_rusanov_n128", "rusanov", "wenojs53", "neumann"),
    ("dirichlet_eo_wenojs32_n100", "eo", "wenojs32", "dirichlet"),
    ("neumann_godunov_constant_n90", "godunov", "constant", "neumann"),
])
def test_step_api_with_boundaries_matches_reference(name, flux_kind, rname, kind):
    """60 steps through ``step()`` with time-dependent boundary data applied at
    the stage times: within 1e-10 of the reference, the same dt sequence."""
    import pyshocks_gb300 as gb

    g = _golden(name)
    n = int(g["n"])
    grid = gb.make_uniform_cell_grid(-1.0, 1.0, n, nghosts=3)
    bc = _bc(kind)
    scheme = gb.bind(_scheme(flux_kind, rname), grid, bc)
    rhs0 = gb.apply_operator(scheme, grid, bc, 0.0, torch.tensor(g["u0"], device="cuda"))
    assert float((rhs0[3:-3].cpu() - torch.tensor(g["rhs0"][3:-3])).abs().max()) < 1.0e-11
    stepper = gb.timestepping.make_time_stepper(scheme, grid, bc, theta=1.0)
    dts, ev = [], None
    for ev in gb.timestepping.step(stepper, torch.tensor(g["u0"], device="cuda"), maxit=60):
        if ev.iteration > 0:
            dts.append(float(ev.dt))
    np.testing.assert_allclose(np.array(dts), g["dts"], rtol=1.0e-12, atol=0)
    err = np.max(np.abs(ev.u.cpu().numpy()[3:-3] - g["u"][3:-3]))
    assert err < 1.0e-10, err


@pytest.mark.parametrize("kind", ["dirichlet", "neumann"])
def test_apply_operator_with_boundary_matches_oracle(kind):
    import pyshocks_gb300 as gb

    n, t = 777, 0.37
    rng = np.random.default_rng(3)
    og = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
    u0 = R.random_fourier_ic(rng, og.f)
    spec = R.SchemeSpec(flux_kind="rusanov", rec="wenojs53", eps=1.0e-6)
    if kind == "dirichlet":
        def obc(tt, u):
            return R.apply_boundary_dirichlet(u, og, tt, dirichlet_np, dirichlet_np)
    else:
        def obc(tt, u):
            return R.apply_boundary_neumann(u, og, tt, neumann_left, neumann_right)
    ref = R.apply_operator(spec, og, u0, t, obc)
    grid = gb.make_uniform_cell_grid(-1.0, 1.0, n, nghosts=3)
    bc = _bc(kind)
    scheme = gb.bind(_scheme("rusanov", "wenojs53"), grid, bc)
    out = gb.apply_operator(scheme, grid, bc, t, torch.tensor(u0, device="cuda")).cpu().numpy()
    err = np.max(np.abs(out[3:-3] - ref[3:-3])) / np.max(np.abs(ref[3:-3]))
    assert err < 1.0e-12, err
    np.testing.assert_array_equal(out[:3], 0.0)


@pytest.mark.parametrize("kind", ["dirichlet", "neumann"])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_batched_plan_with_boundary_matches_oracle(kind, dtype):
    """Uneven instances (one smaller than a tile, one spanning several) with
    constant boundary data per instance, against the oracle stepping each
    instance with the plan's dt sequence."""
    from pyshocks_gb300.batched import BatchedSolver

    sizes = [70, 1500, 2600]
    rng = np.random.default_rng(8)
    u0s = [R.random_fourier_ic(rng, np.linspace(-1, 1, n + 1)) for n in sizes]
    B = len(sizes)
    dvals = np.array([[[0.3, 0.3, 0.3], [-0.2, -0.2, -0.2]],
                      [[0.5, 0.5, 0.5], [0.1, 0.1, 0.1]],
                      [[-0.4, -0.4, -0.4], [0.7, 0.7, 0.7]]])
    nvals = np.array([[0.2, -0.1], [0.0, 0.0], [-0.3, 0.25]])
    scheme = _scheme("rusanov", "wenojs53")
    s = BatchedSolver(scheme, sizes, [2.0 / n for n in sizes], dtype=dtype, max_steps=30)
    if kind == "dirichlet":
        s.set_boundary("dirichlet", dirichlet=dvals)
    else:
        s.set_boundary("neumann", neumann=nvals)
    s.reset(torch.tensor(np.concatenate(u0s)))
    s.step(30)
    assert s.status() == 0
    dts = s.dt_history().cpu().numpy()
    spec = R.SchemeSpec(flux_kind="rusanov", rec="wenojs53", eps=1.0e-6)
    tol = 1.0e-11 if dtype == torch.float64 else 2.0e-4
    for b, n in enumerate(sizes):
        og = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
        if kind == "dirichlet":
            def obc(tt, u, b=b):
                return R.apply_boundary_dirichlet(u, og, tt, lambda t_, x: dvals[b, 0, 0] + 0 * x,
                                                  lambda t_, x: dvals[b, 1, 0] + 0 * x)
        else:
            def obc(tt, u, b=b):
                return R.apply_boundary_neumann(u, og, tt, lambda t_: nvals[b, 0],
                                                lambda t_: nvals[b, 1])
        u = np.concatenate([np.zeros(3), u0s[b], np.zeros(3)])
        u = u.astype(np.float32).astype(np.float64) if dtype == torch.float32 else u
        for k in range(30):
            u = R.ssprk33(lambda tt, v: R.apply_operator(spec, og, v, tt, obc), dts[k, b], 0.0, u)
        got = s.instance(b).double().cpu().numpy()
        err = np.max(np.abs(got - u[3:-3]))
        assert err < tol, (b, err)


@pytest.mark.parametrize("kind", ["dirichlet", "neumann"])
def test_batched_adjoint_with_boundary_against_finite_differences(kind):
    """The exact transpose of the boundary in the batched checkpointed adjoint:
    dJ/du0 . v against central differences of J with the dt sequence replayed
    (two instances, one smaller than a tile)."""
    from pyshocks_gb300.adjoint import CheckpointedSolve
    from pyshocks_gb300.batched import BatchedSolver

    sizes, nsteps = [200, 1300], 24
    x = [np.linspace(-1, 1, n + 1)[:-1] + 1.0 / n for n in sizes]
    u0 = torch.tensor(np.concatenate([0.6 + 0.25 * np.sin(np.pi * xx) + 0.1 * np.cos(3 * np.pi * xx)
                                      for xx in x]), device="cuda")
    rng = np.random.default_rng(4)
    tgt = u0 + 0.05 * torch.tensor(rng.standard_normal(u0.numel()), device="cuda")
    scheme = _scheme("rusanov", "wenojs53")
    dvals = [[0.7, 0.55], [0.4, 0.8]]
    nvals = [[0.2, -0.1], [-0.3, 0.25]]

    def solver():
        s = BatchedSolver(scheme, sizes, [2.0 / n for n in sizes], max_steps=nsteps)
        if kind == "dirichlet":
            d = np.array(dvals)[:, :, None].repeat(3, axis=2)
            s.set_boundary("dirichlet", dirichlet=d)
        else:
            s.set_boundary("neumann", neumann=nvals)
        return s

    s = solver()
    cs = CheckpointedSolve(s, nsteps, stride=5)
    uT = cs.forward(u0).clone()
    g = cs.backward(uT - tgt).clone()
    dts = s.dt_history().clone()

    def J(u):
        s2 = solver()
        s2.set_fixed_dt(dts)
        uT2 = CheckpointedSolve(s2, nsteps).forward(u)
        return 0.5 * float(torch.sum((uT2 - tgt) ** 2))

    assert abs(J(u0) - 0.5 * float(torch.sum((uT - tgt) ** 2))) < 1.0e-12
    h = 1.0e-6
    for k in range(3):
        v = torch.tensor(rng.standard_normal(u0.numel()), device="cuda")
        fd = (J(u0 + h * v) - J(u0 - h * v)) / (2 * h)
        ad = float(torch.dot(g, v))
        # 1e-5: the bar of the periodic test (the Rusanov max(|u_j|, |u_j+1|)
        # switches near extrema within +-h v)
        assert abs(fd - ad) < 1.0e-5 * max(1.0, abs(ad)), (k, fd, ad)


@pytest.mark.parametrize("kind", ["dirichlet", "neumann"])
def test_single_step_vjp_with_boundary_against_finite_differences(kind):
    """``vjp_step`` with time-dependent boundary data (ghosted single
    instance): the transpose of one step against central differences."""
    import pyshocks_gb300 as gb
    from pyshocks_gb300 import burgers
    from pyshocks_gb300.adjoint import vjp_step

    n, t, dt = 300, 0.4, 2.0e-3
    grid = gb.make_uniform_cell_grid(-1.0, 1.0, n, nghosts=3)
    bc = _bc(kind)
    scheme = gb.bind(_scheme("rusanov", "wenojs53"), grid, bc)
    xg = grid.x
    u = (0.6 + 0.25 * torch.sin(np.pi * xg) + 0.1 * torch.cos(3 * np.pi * xg)).contiguous()
    rng = np.random.default_rng(6)
    p = torch.zeros_like(u)
    p[3:-3] = torch.tensor(rng.standard_normal(n), device="cuda")
    g = vjp_step(scheme, grid, dt, u, p, bc=bc, t=t)

    def J(v):
        out = burgers.ssprk33_step(scheme, grid, bc, dt, v, t=t)
        return float(torch.dot(out[3:-3], p[3:-3]))

    # h = 1e-7: the WENO weights ~ 1/(eps + beta)^2 at beta ~ (dx u')^2 make
    # J''' ~ 1e8, so the h^2/6 truncation of h = 1e-6 is ~1e-5 of the gradient
    h = 1.0e-7
    for k in range(3):
        w = torch.zeros_like(u)
        w[3:-3] = torch.tensor(rng.standard_normal(n), device="cuda")
        fd = (J(u + h * w) - J(u - h * w)) / (2 * h)
        ad = float(torch.dot(g[3:-3], w[3:-3]))
        assert abs(fd - ad) < 2.0e-7 * max(1.0, abs(ad)), (k, fd, ad)


def _ghost_table(sizes, dts, nsteps, fn):
    """[nsteps][3][B][2][3] Dirichlet ghost values fn(t, x) at the stage times
    t, t + dt, t + dt/2 of each step; ghost k = 0 is next to the interior."""
    table = np.zeros((nsteps, 3, len(sizes), 2, 3))
    for b, n in enumerate(sizes):
        h = 2.0 / n
        xl = -1.0 - (np.arange(3) + 0.5) * h
        xr = 1.0 + (np.arange(3) + 0.5) * h
        t = 0.0
        for k in range(nsteps):
            for s, ts in enumerate((t, t + dts[b], t + 0.5 * dts[b])):
                table[k, s, b, 0] = fn(ts, xl)
                table[k, s, b, 1] = fn(ts, xr)
            t += dts[b]
    return table


def test_batched_plan_with_time_dependent_dirichlet_matches_oracle():
    """Per-step, per-stage Dirichlet tables (the exact solution of linear
    advection at the ghost centres and stage times) with prescribed steps,
    against the oracle stepping each instance with the same data."""
    from pyshocks_gb300 import burgers, reconstruction
    from pyshocks_gb300.batched import BatchedSolver

    sizes, nsteps = [70, 1500, 600], 25

    def exact(t, x):
        return 0.5 + np.sin(np.pi * (x - t))

    dts = [0.4 * 2.0 / n for n in sizes]
    scheme = burgers.AdvectionRusanov(rec=reconstruction.WENOJS53(eps=1.0e-6))
    s = BatchedSolver(scheme, sizes, [2.0 / n for n in sizes])
    s.set_fixed_dt(np.tile(np.array(dts), (nsteps, 1)))
    s.set_boundary_steps("dirichlet", dirichlet=_ghost_table(sizes, dts, nsteps, exact))
    u0s = []
    for n in sizes:
        f = np.linspace(-1.0, 1.0, n + 1)
        u0s.append(0.5 + (np.cos(np.pi * f[:-1]) - np.cos(np.pi * f[1:])) / (np.pi * (2.0 / n)))
    s.reset(torch.tensor(np.concatenate(u0s)))
    s.step(nsteps)
    assert s.status() == 0
    spec = R.SchemeSpec(flux_kind="rusanov", rec="wenojs53", eps=1.0e-6, equation="advection")
    for b, n in enumerate(sizes):
        og = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)

        def obc(tt, u):
            return R.apply_boundary_dirichlet(u, og, tt, exact, exact)

        u = np.concatenate([np.zeros(3), u0s[b], np.zeros(3)])
        t = 0.0
        for k in range(nsteps):
            u = R.ssprk33(lambda tt, v: R.apply_operator(spec, og, v, tt, obc), dts[b], t, u)
            t += dts[b]
        err = np.max(np.abs(s.instance(b).cpu().numpy() - u[3:-3]))
        assert err < 1.0e-12, (b, err)


def test_batched_adjoint_with_time_dependent_dirichlet_against_finite_differences():
    """The reverse sweep reads each step's boundary row: dJ/du0 . v against
    central differences with per-step Dirichlet tables and prescribed steps."""
    from pyshocks_gb300.adjoint import CheckpointedSolve
    from pyshocks_gb300.batched import BatchedSolver

    sizes, nsteps = [200, 1300], 24
    dts = [0.4 * 2.0 / n for n in sizes]
    table = _ghost_table(sizes, dts, nsteps, lambda t, x: 0.6 + 0.3 * np.sin(np.pi * (x - t)))
    x = [np.linspace(-1, 1, n + 1)[:-1] + 1.0 / n for n in sizes]
    u0 = torch.tensor(np.concatenate([0.6 + 0.25 * np.sin(np.pi * xx) for xx in x]), device="cuda")
    rng = np.random.default_rng(6)
    tgt = u0 + 0.05 * torch.tensor(rng.standard_normal(u0.numel()), device="cuda")
    scheme = _scheme("rusanov", "wenojs53")

    def solver():
        s = BatchedSolver(scheme, sizes, [2.0 / n for n in sizes], max_steps=nsteps)
        s.set_fixed_dt(np.tile(np.array(dts), (nsteps, 1)))
        s.set_boundary_steps("dirichlet", dirichlet=table)
        return s

    s = solver()
    cs = CheckpointedSolve(s, nsteps, stride=5)
    uT = cs.forward(u0).clone()
    g = cs.backward(uT - tgt).clone()

    def J(u):
        uT2 = CheckpointedSolve(solver(), nsteps).forward(u)
        return 0.5 * float(torch.sum((uT2 - tgt) ** 2))

    h = 1.0e-6
    for k in range(3):
        v = torch.tensor(rng.standard_normal(u0.numel()), device="cuda")
        fd = (J(u0 + h * v) - J(u0 - h * v)) / (2 * h)
        ad = float(torch.dot(g, v))
        assert abs(fd - ad) < 1.0e-5 * max(1.0, abs(ad)), (k, fd, ad)
