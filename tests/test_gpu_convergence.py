"""Orders of convergence of the GPU path: the reference's property tests
(``tests/test_convergence.py``) run through batched plans with prescribed
steps. The advection study runs every resolution as one instance of a single
batch (uneven sizes, a dt table per instance)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import numpy_ref as R

pytestmark = pytest.mark.gpu


def _eoc(hs, errs):
    return R.estimate_order_of_convergence(np.asarray(hs), np.asarray(errs))


def _dt_table(dts, maxits):
    """(max maxit, B) prescribed steps: instance b takes maxits[b] steps of
    dts[b], then steps of 0 (no change)."""
    table = np.zeros((max(maxits), len(dts)))
    for b, (dt, m) in enumerate(zip(dts, maxits)):
        table[:m, b] = dt
    return table


def _run(scheme, sizes, a, b, u0, table, *, boundary=None):
    from pyshocks_gb300.batched import BatchedSolver

    dx = [(b - a) / n for n in sizes]
    s = BatchedSolver(scheme, sizes, dx)
    if boundary is not None:
        s.set_boundary("dirichlet", dirichlet=boundary)
    s.set_fixed_dt(table)
    s.reset(torch.tensor(np.concatenate(u0), device="cuda"))
    s.step(table.shape[0])
    assert s.status() == 0
    return [s.instance(i).double().cpu().numpy() for i in range(len(sizes))]


def test_advection_convergence_wenojs53_gpu():
    """``tests/test_convergence.py:395-460``: periodic linear advection (a = 1),
    WENOJS53 (eps 1e-12) with the upwind flux (Rusanov at constant speed),
    SSPRK33 with dt = 8 h^{5/3}, EOC >= 4.5 in the weighted relative L1 norm."""
    from pyshocks_gb300 import burgers, grid as G, reconstruction

    sizes = list(range(32, 256 + 1, 32))
    scheme = burgers.AdvectionRusanov(rec=reconstruction.WENOJS53(eps=1.0e-12))
    u0, exact, dts, maxits, hs = [], [], [], [], []
    tfinal = 1.0
    for n in sizes:
        g = G.make_uniform_cell_grid(-1.0, 1.0, n, nghosts=3)
        og = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
        q = G.make_leggauss_quadrature(g, order=5)
        u0.append(G.cell_average(q, lambda x: R.ic_sine_sine(og, x))[3:-3])
        exact.append(G.cell_average(q, lambda x: R.ic_sine_sine(og, x - tfinal))[3:-3])
        dt = 8.0 * (2.0 / n) ** (5.0 / 3.0)
        maxit = int(tfinal / dt)
        dts.append(tfinal / maxit + 1.0e-15)
        maxits.append(maxit)
        hs.append(2.0 / n)
    out = _run(scheme, sizes, -1.0, 1.0, u0, _dt_table(dts, maxits))
    errs = [np.sum(np.abs(u - e)) / np.sum(np.abs(e)) for u, e in zip(out, exact)]
    assert _eoc(hs, errs) >= 4.5, errs


@pytest.mark.parametrize(("name", "sizes"), [
    ("rusanov", list(range(64, 128 + 1, 16))),
    ("eo", list(range(32, 128 + 1, 16))),
])
def test_burgers_riemann_convergence_gpu(name, sizes):
    """``tests/test_convergence.py:222-303``: the Burgers Riemann problem
    (u_L = 1, u_R = 0, shock from x = 0 at speed 1/2) on [-1, 1] with Dirichlet
    data from the exact solution, constant reconstruction, Rusanov with
    alpha = 0.98 (and Engquist-Osher), SSPRK33 with the dt of
    predict_timestep_from_resolutions (umax 10) to t = 1, first order
    (EOC >= 0.9) in the weighted relative L1 norm."""
    from pyshocks_gb300 import burgers, grid as G, reconstruction

    rec = reconstruction.ConstantReconstruction()
    scheme = (burgers.Rusanov(rec=rec, alpha=0.98) if name == "rusanov"
              else burgers.EngquistOsher(rec=rec))
    from pyshocks_gb300 import timestepping as ts

    tfinal = 1.0
    maxit, dt = ts.predict_maxit_from_timestep(
        tfinal, ts.predict_timestep_from_resolutions(-1.0, 1.0, sizes, umax=10.0))

    def riemann(t):
        return lambda x: np.where(x < 0.5 * t, 1.0, 0.0)

    u0, exact = [], []
    for n in sizes:
        g = G.make_uniform_cell_grid(-1.0, 1.0, n, nghosts=3)
        q = G.make_leggauss_quadrature(g, order=5)
        u0.append(G.cell_average(q, riemann(0.0))[3:-3])
        exact.append(G.cell_average(q, riemann(tfinal))[3:-3])
    # ghost values: u_L on the left (x < -1), u_R on the right, at every stage
    bnd = np.zeros((1, 2, 3))
    bnd[:, 0, :] = 1.0
    table = np.full((maxit, 1), dt)
    # one plan per resolution: Rusanov's nu = dx^(alpha - 1) is one value per plan
    out = [_run(scheme, [n], -1.0, 1.0, [v], table, boundary=bnd)[0] for n, v in zip(sizes, u0)]
    hs = [2.0 / n for n in sizes]
    errs = [np.sum(np.abs(u - e)) / np.sum(np.abs(e)) for u, e in zip(out, exact)]
    assert _eoc(hs, errs) >= 1 - 0.1, errs


def test_rusanov_alpha_plan_needs_one_dx():
    """nu = dx^(alpha - 1) is one value per plan: mixed cell sizes are refused."""
    from pyshocks_gb300 import burgers, reconstruction
    from pyshocks_gb300.batched import BatchedSolver

    scheme = burgers.Rusanov(rec=reconstruction.ConstantReconstruction(), alpha=0.98)
    with pytest.raises(ValueError, match="share dx"):
        BatchedSolver(scheme, [64, 128], [2.0 / 64, 2.0 / 128])
    BatchedSolver(scheme, [64, 64], 2.0 / 64)  # one dx: fine


def test_ssprk33_time_order_gpu():
    """``tests/test_timestepping.py:26-99`` on the GPU path: SSPRK33 is third
    order in time. One batch of the same grid (periodic advection, N = 256,
    WENOJS53) stepped to t = 1 with Courant numbers 0.8, 0.4, 0.2, 0.1 and a
    reference at 0.0125: the spatial error is common to all instances, so the
    differences to the reference are the temporal errors."""
    from pyshocks_gb300 import burgers, grid as G, reconstruction

    n, tfinal = 256, 1.0
    h = 2.0 / n
    scheme = burgers.AdvectionRusanov(rec=reconstruction.WENOJS53(eps=1.0e-6))
    g = G.make_uniform_cell_grid(-1.0, 1.0, n, nghosts=3)
    q = G.make_leggauss_quadrature(g, order=5)
    v0 = G.cell_average(q, lambda x: np.sin(np.pi * x))[3:-3]
    courant = [0.8, 0.4, 0.2, 0.1, 0.0125]
    maxits = [int(np.ceil(tfinal / (c * h))) for c in courant]
    dts = [tfinal / m for m in maxits]
    out = _run(scheme, [n] * len(courant), -1.0, 1.0, [v0] * len(courant), _dt_table(dts, maxits))
    ref = out[-1]
    errs = [np.sum(np.abs(u - ref)) * h for u in out[:-1]]
    assert _eoc(dts[:-1], errs) >= 3 - 0.1, errs
