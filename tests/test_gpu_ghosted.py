"""The reference's step on one ghosted array (``shk_*_ghosted_f64``): forward
against the NumPy oracle on every cell, ghost outputs included; the exact
transpose against ``torch.func.vjp`` of the ghosted torch restatement (the
stand-in for ``jax.jacfwd`` in ``src/pyshocks/timestepping.py:174``, pinned to
the NumPy oracle by ``tests/test_oracle.py``); and the reference adjoint
driver (``drivers/burgers-adjoint.py``: global Lax-Friedrichs, alpha 0.995,
constant reconstruction on a one-ghost grid, Dirichlet forward boundary,
homogeneous Neumann adjoint boundary, p0 = u(T)) end to end through ``step``
and ``adjoint_step``; and, for a linear scheme, the transpose against the
whole finite-difference Jacobian of the forward step (the reference's
``tests/test_finite_difference.py`` check).

Tolerances: operator and step 1e-12 relative to the data scale (different
summation order, and (2k+1) dx for the Neumann mirror distance where the
oracle subtracts cell centres); one transposed step 1e-11 relative; the
driver's 100+ step adjoint 1e-9 relative.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from oracle import numpy_ref as R
from oracle import torch_ref as T

pytestmark = pytest.mark.gpu

CASES = [(rec, fk, alpha, kind, g)
         for rec, g in (("constant", 1), ("constant", 3), ("wenojs53", 3))
         for fk, alpha in (("rusanov", 1.0), ("rusanov", 0.98), ("lf", 1.0), ("lf", 0.995))
         for kind in ("periodic", "dirichlet", "neumann")]


def _c_args(L, rec, fk, alpha, tb, g, dx):
    s = L.ShkScheme(flux=L.SHK_FLUX_LF if fk == "lf" else L.SHK_FLUX_RUSANOV,
                    rec=L.SHK_REC_CONSTANT if rec == "constant" else L.SHK_REC_WENOJS53,
                    equation=L.SHK_EQ_BURGERS, eps=1.0e-6, delta=0.0,
                    nu=1.0 if alpha == 1.0 else dx ** (alpha - 1), speed=1.0)
    b = L.ShkBoundary()
    kinds = {"periodic": L.SHK_BC_PERIODIC, "dirichlet": L.SHK_BC_DIRICHLET,
             "neumann": L.SHK_BC_NEUMANN}
    b.left, b.right = kinds[tb["left"]], kinds[tb["right"]]
    for st in range(3):
        for side in range(2):
            b.neumann[st * 2 + side] = float(tb["neumann"][st][side])
            for k in range(3):
                b.dirichlet[(st * 2 + side) * 3 + k] = float(tb["dirichlet"][st][side][k])
    return s, b


def _ws(L, n, g):
    return torch.empty(int(L.lib().shk_ghosted_workspace_bytes(n, g)), dtype=torch.uint8,
                       device="cuda")


@pytest.mark.parametrize(("rec", "fk", "alpha", "kind", "g"), CASES)
def test_ghosted_operator_and_step_match_oracle(rec, fk, alpha, kind, g):
    from test_oracle import _ghosted_case

    from pyshocks_gb300 import _lib as L

    grid, u, spec, tb, bc, times, dt = _ghosted_case(rec, fk, alpha, kind, g)
    n = grid.x.size - 2 * g
    s, b = _c_args(L, rec, fk, alpha, tb, g, grid.dx_min)
    ws = _ws(L, n, g)
    ud = torch.tensor(u, device="cuda")
    out = torch.empty_like(ud)
    st = L.lib().shk_apply_operator_ghosted_f64(s, ctypes.byref(b), ud.data_ptr(), out.data_ptr(),
                                                n, g, grid.dx_min, ws.data_ptr(), ws.numel(),
                                                L.stream_handle())
    assert st == 0, L.errstr(st)
    ref = R.apply_operator(spec, grid, u, times[0], bc)
    assert np.max(np.abs(out.cpu().numpy() - ref)) <= 1.0e-12 * np.max(np.abs(ref))
    st = L.lib().shk_ssprk33_step_ghosted_f64(s, ctypes.byref(b), ud.data_ptr(), out.data_ptr(),
                                              n, g, grid.dx_min, dt, ws.data_ptr(), ws.numel(),
                                              L.stream_handle())
    assert st == 0, L.errstr(st)
    ref = R.ssprk33(lambda t, v: R.apply_operator(spec, grid, v, t, bc), dt, times[0], u)
    assert np.max(np.abs(out.cpu().numpy() - ref)) <= 1.0e-12 * np.max(np.abs(ref))


def _plateau(grid):
    """A state whose maximum |u| is attained by many cells (a plateau) and by
    ghost cells: the global Lax-Friedrichs speed ties across all of them."""
    x = grid.x
    return np.where(np.abs(x) < 0.5, 1.0, 0.25 * np.sin(np.pi * x))


@pytest.mark.parametrize(("rec", "fk", "alpha", "kind", "g"), CASES)
@pytest.mark.parametrize("state", ["fourier", "plateau"])
def test_ghosted_vjp_matches_autograd(rec, fk, alpha, kind, g, state):
    """J^T p of one ghosted step with a cotangent that is nonzero on the ghost
    cells too, against torch.func.vjp of the ghosted restatement."""
    from test_oracle import _ghosted_case

    from pyshocks_gb300 import _lib as L

    grid, u, spec, tb, bc, times, dt = _ghosted_case(rec, fk, alpha, kind, g)
    if state == "plateau":
        u = _plateau(grid)
    n = grid.x.size - 2 * g
    nu = 1.0 if alpha == 1.0 else grid.dx_min ** (alpha - 1)
    p = np.random.default_rng(11).standard_normal(u.size)
    ref = T.ghosted_step_vjp(torch.tensor(u), torch.tensor(p), dt, grid.dx_min, g, tb,
                             torch.tensor(grid.x), rec=rec, flux_kind=fk, eps=1.0e-6,
                             nu=nu).numpy()
    s, b = _c_args(L, rec, fk, alpha, tb, g, grid.dx_min)
    ws = _ws(L, n, g)
    ud = torch.tensor(u, device="cuda")
    pd = torch.tensor(p, device="cuda")
    out = torch.empty_like(ud)
    st = L.lib().shk_ssprk33_vjp_ghosted_f64(s, ctypes.byref(b), ud.data_ptr(), pd.data_ptr(),
                                             out.data_ptr(), n, g, grid.dx_min, dt, ws.data_ptr(),
                                             ws.numel(), L.stream_handle())
    assert st == 0, L.errstr(st)
    got = out.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1.0e-11 * np.max(np.abs(ref)), np.max(np.abs(got - ref))


def _tophat(grid_a, grid_b, t, x):
    """The rarefaction-shock solution of the reference driver's initial
    condition (``src/pyshocks/funcs.py:426-474``, us = 0, uc = 1, the top hat on
    the middle half of the domain)."""
    xm, L_ = (grid_b + grid_a) / 2, grid_b - grid_a
    xa, xb = xm - 0.25 * L_, xm + 0.25 * L_
    us, uc = 0.0, 1.0
    s = (uc + us) / 2

    def ind(c):
        return c.double() if isinstance(c, torch.Tensor) else c.astype(np.float64)

    h_l = ind(x < xa + us * t)
    h_e = ind((xa + us * t < x) & (x < xa + uc * t))
    h_c = ind((xa + uc * t < x) & (x < xb + s * t))
    h_r = ind(x > xb + s * t)
    return us * h_l + (x - xa) / (t + 1.0e-15) * h_e + uc * h_c + us * h_r


@pytest.mark.parametrize("ic", ["tophat", "smooth"])
def test_reference_adjoint_driver_end_to_end(ic):
    """``drivers/burgers-adjoint.py`` (its defaults: n = 256 on [-1.5, 1.5],
    t_final = 0.75, theta = 1, ``lf`` with alpha = 0.995 and the default
    constant reconstruction, so one ghost cell; Dirichlet forward boundary),
    ``step`` to t_final with in-memory checkpoints, then ``adjoint_step`` from
    p0 = u(T) with the homogeneous Neumann adjoint boundary applied to p after
    each step. Compared with the same loop on the ghosted torch restatement
    (torch.func.vjp per step, at the GPU's checkpointed states and dt).

    ``tophat``: the driver's own initial state (cell averages of the top hat by
    2-point Gauss-Legendre, Dirichlet data from the exact solution). Its
    maximum |u| = 1 is attained on a whole plateau, so the Lax-Friedrichs
    speed's cotangent is split among the tied cells, and whether a cell at the
    plateau's edge rounds to exactly 1 in the recomputed stage states depends
    on the arithmetic's rounding (the reference's XLA order has its own).
    The tie count then differs by a cell here and there: a few entries move by
    up to ~1e-4, the rest agree to round-off (measured: max 6.8e-5, mean 4.8e-6
    of the range). Bar: 1e-3 of the range in max-abs, 2e-5 in the mean.

    ``smooth``: the same pipeline from a smooth state with a single maximum
    (constant Dirichlet data): 1e-9 relative. There the ghost rows matter: the
    interior-only transpose (ghost cotangents dropped before each step) is off
    by O(1), and the GPU result must be far from it."""
    import pyshocks_gb300 as gb
    from pyshocks_gb300 import burgers, reconstruction, scalar
    from pyshocks_gb300.checkpointing import InMemoryCheckpoint
    from pyshocks_gb300.grid import cell_average, make_leggauss_quadrature

    a, b, n, tfinal = -1.5, 1.5, 256, 0.75
    rec = reconstruction.make_reconstruction_from_name("default")
    scheme = burgers.make_scheme_from_name("lf", rec=rec, alpha=0.995)
    assert rec.stencil_width == 1
    grid = gb.make_uniform_cell_grid(a=a, b=b, n=n, nghosts=scheme.stencil_width)
    g = grid.nghosts
    x = grid.x.double().cpu()
    if ic == "tophat":
        quad = make_leggauss_quadrature(grid, order=int(max(scheme.order, 1)) + 1)
        u0 = cell_average(quad, lambda xx: _tophat(a, b, 0.0, xx), like=grid.x)

        def gfun(t, xx):
            return _tophat(a, b, t, xx)
    else:
        u0 = (0.5 + 0.4 * torch.sin(np.pi * grid.x / 1.5)
              + 0.1 * torch.cos(2 * np.pi * grid.x / 1.5)).double().contiguous()
        vl, vr = float(u0[0]), float(u0[-1])

        def gfun(t, xx):
            out = torch.full_like(torch.as_tensor(xx, dtype=torch.float64), vl)
            out[torch.as_tensor(xx) > 0] = vr
            return out
    bc = scalar.make_dirichlet_boundary(ga=gfun)
    scheme = gb.bind(scheme, grid, bc)
    stepper = gb.timestepping.make_time_stepper(scheme, grid, bc, theta=1.0,
                                                checkpoint=InMemoryCheckpoint("Iteration"))
    dts, states = [], [u0.clone()]
    for ev in gb.timestepping.step(stepper, u0, tfinal=tfinal):
        if ev.iteration > 0:
            dts.append(ev.dt)
            states.append(ev.u.clone())
    uf, maxit = ev.u, ev.iteration
    assert maxit > 100
    nbc = scalar.make_neumann_boundary(lambda t: 0.0)

    def adj_bc(t, u, p):
        return gb.apply_boundary(nbc, grid, t, p)

    for ev in gb.timestepping.adjoint_step(stepper, uf, maxit=maxit, apply_boundary=adj_bc):
        pass
    got = ev.p.cpu().numpy()

    # the same loop on the ghosted restatement (CPU, float64)
    xg = x[torch.tensor([0, g + n])]
    nu = grid.dx_min ** (0.995 - 1)
    # checkpoint times as step() accumulates them; the adjoint's dt is their
    # difference (timestepping.py:200-201)
    t = 0.0
    times = [t]
    for dt in dts:
        t += dt
        times.append(t)

    def table(t0, dt):
        d = np.zeros((3, 2, 3))
        for s_, ts in enumerate((t0, t0 + dt, t0 + 0.5 * dt)):
            v = gfun(ts, xg)
            d[s_, 0, 0], d[s_, 1, 0] = float(v[0]), float(v[1])
        return {"left": "dirichlet", "right": "dirichlet", "dirichlet": d,
                "neumann": np.zeros((3, 2))}

    def neumann0(p):
        p = p.clone()
        p[:g] = p[g:2 * g].flip(0)
        p[p.shape[0] - g:] = p[p.shape[0] - 2 * g:p.shape[0] - g].flip(0)
        return p

    def sweep(interior_only):
        p = neumann0(uf.double().cpu())
        for m in range(maxit - 1, -1, -1):
            dt = times[m + 1] - times[m]
            if interior_only:
                p = p.clone()
                p[:g] = 0.0
                p[p.shape[0] - g:] = 0.0
            p = T.ghosted_step_vjp(states[m].double().cpu(), p, dt, grid.dx_min, g,
                                   table(times[m], dt), x, rec="constant", flux_kind="lf", nu=nu)
            p = neumann0(p)
        return p.numpy()

    ref = sweep(False)
    scale = np.max(np.abs(ref))
    assert scale > 0.1
    d = np.abs(got - ref)
    if ic == "tophat":
        assert np.max(d) <= 1.0e-3 * scale, np.max(d)
        assert np.mean(d) <= 2.0e-5 * scale, np.mean(d)
    else:
        assert np.max(d) <= 1.0e-9 * scale, np.max(d)
        assert np.max(np.abs(got - sweep(True))) > 0.1 * scale


@pytest.mark.parametrize("kind", ["periodic", "dirichlet"])
def test_linear_step_transpose_matches_finite_difference_jacobian(kind):
    """The reference's finite-difference check of a linear scheme's Jacobian
    (``tests/test_finite_difference.py:110-171``: constant reconstruction,
    periodic or zero Dirichlet data, n = 32, central differences of every
    component) on the ghosted GPU step: linear advection (c = 1) with the
    Rusanov flux and the constant reconstruction is linear in u, so central
    differences of the forward step give its whole Jacobian, ghost rows and
    columns included, up to rounding, and the matrix-free transpose applied to
    every unit cotangent must give its transpose. Bars: at the reference's
    eps = 1e-3 the float64 rounding of the two steps divided by 2 eps is the
    floor (the torch restatement itself lands at 1.0e-13 there), so 5e-13; at
    eps = 1 (exact for a linear map) 1e-14 (the restatement: 1.3e-16)."""
    from pyshocks_gb300 import _lib as L

    n, g = 32, 1
    dx = 2.0 / n
    dt = 0.5 * dx
    m = n + 2 * g
    s = L.ShkScheme(flux=L.SHK_FLUX_RUSANOV, rec=L.SHK_REC_CONSTANT, equation=L.SHK_EQ_ADVECTION,
                    eps=1.0e-6, delta=0.0, nu=1.0, speed=1.0)
    b = L.ShkBoundary()
    b.left = b.right = L.SHK_BC_PERIODIC if kind == "periodic" else L.SHK_BC_DIRICHLET
    ws = _ws(L, n, g)
    u = np.random.default_rng(42).standard_normal(m)

    def step(v):
        vd = torch.tensor(v, device="cuda")
        out = torch.empty_like(vd)
        st = L.lib().shk_ssprk33_step_ghosted_f64(s, ctypes.byref(b), vd.data_ptr(), out.data_ptr(),
                                                  n, g, dx, dt, ws.data_ptr(), ws.numel(),
                                                  L.stream_handle())
        assert st == 0, L.errstr(st)
        return out.cpu().numpy()

    ud = torch.tensor(u, device="cuda")
    jt = np.empty((m, m))
    for i in range(m):
        pd = torch.zeros(m, dtype=torch.float64, device="cuda")
        pd[i] = 1.0
        out = torch.empty_like(ud)
        st = L.lib().shk_ssprk33_vjp_ghosted_f64(s, ctypes.byref(b), ud.data_ptr(), pd.data_ptr(),
                                                 out.data_ptr(), n, g, dx, dt, ws.data_ptr(),
                                                 ws.numel(), L.stream_handle())
        assert st == 0, L.errstr(st)
        jt[:, i] = out.cpu().numpy()  # column i of J^T = row i of J
    for eps, bar in ((1.0e-3, 5.0e-13), (1.0, 1.0e-14)):
        fd = np.empty((m, m))
        for i in range(m):
            e = np.zeros(m)
            e[i] = eps
            fd[:, i] = (step(u + e) - step(u - e)) / (2.0 * eps)
        err = np.linalg.norm(jt.T - fd) / np.linalg.norm(fd)
        assert err < bar, (eps, err)
