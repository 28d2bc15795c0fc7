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


def test_adjoint_refuses_non_periodic_plans():
    from pyshocks_gb300.adjoint import CheckpointedSolve
    from pyshocks_gb300.batched import BatchedSolver

    s = BatchedSolver(_scheme("rusanov", "wenojs53"), [256], 2.0 / 256, max_steps=4)
    s.set_boundary("neumann", neumann=[0.0, 0.0])
    cs = CheckpointedSolve(s, 4)
    u0 = torch.tensor(0.5 + 0.2 * np.sin(np.linspace(0, 2 * np.pi, 256)), device="cuda")
    uT = cs.forward(u0)
    with pytest.raises(Exception):
        cs.backward(uT.clone())
