"""Pins the oracle (``oracle/numpy_ref.py``, ``oracle/torch_ref.py``) against

* golden vectors produced by the reference's own source
  (``tests/golden/make_golden.py``), and
* the reference's own property tests on this path, ported onto the oracle:
  ``tests/test_weno.py:34-166,288-338``, ``tests/test_timestepping.py:26-99``,
  ``tests/test_convergence.py:395-460``.
"""

from __future__ import annotations

import pathlib
from itertools import product

import numpy as np
import pytest
import torch

from oracle import numpy_ref as R
from oracle import torch_ref as T

GOLDEN = pathlib.Path(__file__).parent / "golden"


def _load(name):
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    g["__name__"] = name
    return g


# {{{ golden vectors from the reference


@pytest.mark.parametrize("name", ["sine", "step"])
@pytest.mark.parametrize("rec", ["wenojs53", "wenojs32", "esweno32"])
def test_recon_golden(name, rec):
    g = _load(f"recon_{name}")
    u = g["u"]
    s = R.weno_js_53_coefficients() if rec == "wenojs53" else R.weno_js_32_coefficients()
    eps = 1.0e-6
    np.testing.assert_array_equal(R.weno_smoothness(s, u), g[f"{rec}_beta"])
    np.testing.assert_array_equal(R.weno_interp(s, u), g[f"{rec}_uhat"])
    if rec == "esweno32":
        omega = R.es_weno_weights(s, u, eps)
        ul, ur = R.reconstruct_esweno32(s, eps, u)
    else:
        omega = R.weno_js_weights(s, u, eps)
        ul, ur = R.reconstruct_wenojs(s, eps, u)
    np.testing.assert_array_equal(omega, g[f"{rec}_omega"])
    np.testing.assert_array_equal(ul, g[f"{rec}_ul"])
    np.testing.assert_array_equal(ur, g[f"{rec}_ur"])


RUNS = [
    ("sine_rusanov_n256", "rusanov", "burgers", {"tfinal": 1.0}),
    ("sine_lf_n256", "lf", "burgers", {"tfinal": 1.0}),
    ("sine_esweno_n256", "esweno", "burgers", {"tfinal": 1.0}),
    ("fourier_rusanov_n64_s11", "rusanov", "burgers", {"maxit": 40}),
    ("fourier_rusanov_n96_s12", "rusanov", "burgers", {"maxit": 40}),
    ("fourier_rusanov_n128_s13", "rusanov", "burgers", {"maxit": 40}),
    ("fourier_rusanov_n50_s14", "rusanov", "burgers", {"maxit": 40}),
    ("fourier_lf_n64_s21", "lf", "burgers", {"maxit": 40}),
    ("fourier_esweno_n64_s22", "esweno", "burgers", {"maxit": 40}),
    ("lwr_rusanov_n128_s31", "rusanov", "lwr", {"maxit": 60}),
    ("sine_godunov_wenojs53_n256", "godunov", "burgers", {"tfinal": 1.0}),
    ("sine_eo_wenojs53_n256", "eo", "burgers", {"tfinal": 1.0}),
] + [(f"fourier_{f}_{r}_n96_s{s}", f, "burgers", {"maxit": 40})
     for f in ("rusanov", "godunov", "eo") for r, s in (("constant", 41), ("wenojs32", 42))]


def _spec(g, flux_kind, equation):
    if flux_kind == "esweno":
        return R.SchemeSpec(flux_kind="esweno", rec="esweno32", eps=float(g["eps"]),
                            delta=float(g["delta"]), equation=equation)
    name = str(g.get("__name__", ""))
    rec = "constant" if "_constant_" in name else ("wenojs32" if "_wenojs32_" in name else "wenojs53")
    return R.SchemeSpec(flux_kind=flux_kind, rec=rec, eps=1.0e-6, equation=equation)


@pytest.mark.parametrize(("name", "flux_kind", "equation", "kw"), RUNS)
def test_numpy_oracle_runs_golden(name, flux_kind, equation, kw):
    g = _load(name)
    n = int(g["n"])
    grid = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
    spec = _spec(g, flux_kind, equation)
    if flux_kind == "esweno":
        eps, delta = R.es_weno_parameters(grid, np.ones_like(grid.x))
        assert eps == float(g["eps"]) and delta == float(g["delta"])
    rhs0 = R.apply_operator(spec, grid, g["u0"])
    # the whole ghosted arrays: the ghost outputs of the operator (zero-padded
    # convolutions and end fluxes) and the ghost values the steps pass through
    np.testing.assert_array_equal(rhs0, g["rhs0"])
    assert R.predict_timestep(spec, grid, g["u0"]) == float(g["dt0"])
    u, dts = R.evolve(spec, grid, g["u0"], theta=1.0, **kw)
    np.testing.assert_array_equal(np.array(dts), g["dts"])
    np.testing.assert_array_equal(u, g["u"])


@pytest.mark.parametrize(("name", "flux_kind", "equation", "kw"), RUNS)
def test_torch_oracle_runs_golden(name, flux_kind, equation, kw):
    """The torch restatement (used for derivatives) follows the reference to
    round-off: same final state within 1e-11 with the reference's dt sequence."""
    g = _load(name)
    n = int(g["n"])
    spec = _spec(g, flux_kind, equation)
    u0 = torch.tensor(g["u0"][3:-3])[None]
    dts = torch.tensor(g["dts"]).reshape(-1, 1)
    u, _ = T.forward(u0, 2.0 / n, len(g["dts"]), dts=dts, flux_kind=flux_kind,
                     rec=spec.rec, eps=spec.eps, delta=spec.delta, equation=equation)
    err = np.max(np.abs(u[0].numpy() - g["u"][3:-3]))
    assert err < 1.0e-11, err


# }}}


# {{{ ports of the reference's property tests


def test_convolve_same_vs_scipy():
    """``tests/test_utils.py:21-86`` compares the reference's ``convolve1d``
    with ``scipy.ndimage.convolve1d`` for its padded modes; the path uses the
    "same" mode (zero padding, ``src/pyshocks/convolve.py:113-114``), which for
    the odd stencil lengths of the reconstructions is scipy's ``constant``
    mode. Random sizes as in the reference test, relative error below 1e-12."""
    snd = pytest.importorskip("scipy.ndimage")
    rng = np.random.default_rng(seed=42)
    for _ in range(16):
        n = int(rng.integers(126, 384))
        m = 2 * int(rng.integers(1, 14)) + 1
        a = rng.random(n)
        w = rng.random(m)
        ref = snd.convolve1d(a, w, mode="constant", cval=0.0)
        got = R.convolve1d(a, w)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1.0e-12, (n, m)


@pytest.mark.parametrize("rec_name", ["wenojs32", "wenojs53"])
def test_weno_smoothness_indicator_vectorization(rec_name):
    """``tests/test_weno.py:34-108``: loop vs convolution, rtol 2e-15."""
    rtol = 2.0e-15
    s = R.weno_js_53_coefficients() if rec_name == "wenojs53" else R.weno_js_32_coefficients()
    nghosts = s.b.shape[-1] // 2
    nstencils = s.b.shape[0]
    stencil = np.arange(-nghosts, nghosts + 1)
    n = 64 + 2 * nghosts
    m = np.s_[nghosts:-nghosts]
    u = np.sin(np.linspace(0.0, 2.0 * np.pi, n))

    beta0 = np.zeros((nstencils, n))
    for j in range(*m.indices(n)):
        for i, k in product(range(nstencils), range(s.a.size)):
            beta0[i, j] += s.a[k] * np.sum(u[j + stencil] * s.b[i, k, ::-1]) ** 2
    beta1 = R.weno_smoothness(s, u)
    uhat0 = np.zeros((nstencils, n))
    for j in range(*m.indices(n)):
        for i in range(nstencils):
            uhat0[i, j] = np.sum(u[j + stencil] * s.c[i, ::-1])
    uhat1 = R.weno_interp(s, u)
    err = np.linalg.norm(beta0[:, m] - beta1[:, m]) / np.linalg.norm(beta0[:, m])
    assert err < rtol
    err = np.linalg.norm(uhat0[:, m] - uhat1[:, m]) / np.linalg.norm(uhat0[:, m])
    assert err < rtol


@pytest.mark.parametrize(("rec_name", "n"), [("wenojs32", 512), ("wenojs53", 128)])
@pytest.mark.parametrize("is_smooth", [True, False])
def test_weno_smoothness_indicator(rec_name, n, is_smooth):
    """``tests/test_weno.py:117-166``."""
    s = R.weno_js_53_coefficients() if rec_name == "wenojs53" else R.weno_js_32_coefficients()
    eps = 1.0e-12 if rec_name == "wenojs53" else 1.0e-6
    nghosts = s.b.shape[-1] // 2
    n = n + 2 * nghosts
    m = np.s_[nghosts:-nghosts]
    theta = np.linspace(0.0, 2.0 * np.pi, n)
    u = np.sin(theta) if is_smooth else (theta < np.pi).astype(np.float64)
    omega = R.weno_js_weights(s, u, eps)
    error = np.max(np.abs(omega[:, m] - s.d))
    if is_smooth:
        assert error < 0.1
    else:
        assert error > 0.1


def test_weno53_smooth_reconstruction_order():
    """``tests/test_weno.py:288-338`` for WENOJS53 (order 5, EOC >= 4.5)."""
    hs, el, er = [], [], []
    s = R.weno_js_53_coefficients()

    def func(x):
        return np.sin(2.0 * np.pi * x)

    for n in range(32, 256 + 1, 32):
        grid = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
        u0 = R.cell_average_leggauss(grid, func, order=6)
        ref = func(grid.f)
        ul, ur = R.reconstruct_wenojs(s, 1.0e-12, u0)
        i = grid.i_
        el.append(np.max(np.abs(ul - ref[:-1])[i]) / np.max(np.abs(ref[:-1][i])))
        er.append(np.max(np.abs(ur - ref[1:])[i]) / np.max(np.abs(ref[1:][i])))
        hs.append(grid.dx_min)
    assert R.estimate_order_of_convergence(np.array(hs), np.array(el)) >= 4.5
    assert R.estimate_order_of_convergence(np.array(hs), np.array(er)) >= 4.5


def test_ssprk33_time_convergence():
    """``tests/test_timestepping.py:26-99`` for SSPRK33: u' = e^{-t}."""
    tfinal = 4.0
    hs, errs = [], []
    for n in range(2, 7):
        dt = 1.0 / 2.0**n
        maxit = int(tfinal / dt)
        dt = tfinal / maxit + 1.0e-15
        u = np.array([-1.0])
        t = 0.0
        for _ in range(maxit):
            u = R.ssprk33(lambda t_, u_: np.array([np.exp(-t_)]), dt, t, u)
            t += dt
        u_ex = -np.exp(-tfinal)
        errs.append(abs(u[0] - u_ex) / abs(u_ex))
        hs.append(dt)
    assert R.estimate_order_of_convergence(np.array(hs), np.array(errs)) >= 3 - 0.1


def test_advection_convergence_wenojs53():
    """``tests/test_convergence.py:395-460``: periodic linear advection (a = 1)
    with WENOJS53 (eps 1e-12) and an upwind flux, SSPRK33, dt = 8 h^{5/3},
    EOC >= 4.5 in the weighted relative L1 norm. For a = 1 > 0 the Rusanov
    flux with a constant speed is the upwind flux."""
    hs, errs = [], []
    for n in range(32, 256 + 1, 32):
        grid = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
        spec = R.SchemeSpec(flux_kind="rusanov", rec="wenojs53", eps=1.0e-12,
                            equation="advection")
        u0 = R.cell_average_leggauss(grid, lambda x: R.ic_sine_sine(grid, x), order=5)
        tfinal = 1.0
        dt = 8.0 * (2.0 / n) ** (5.0 / 3.0)
        maxit = int(tfinal / dt)
        dt = tfinal / maxit + 1.0e-15
        ev = None
        for ev in R.step(lambda t, u: dt, lambda t, u: R.apply_operator(spec, grid, u),
                         u0, maxit=maxit):
            pass
        uhat = R.cell_average_leggauss(grid, lambda x: R.ic_sine_sine(grid, x - tfinal),
                                       order=5)
        err = R.norm(grid, ev.u - uhat, p=1, weighted=True) / R.norm(grid, uhat, p=1,
                                                                     weighted=True)
        hs.append(grid.dx_min)
        errs.append(err)
    assert R.estimate_order_of_convergence(np.array(hs), np.array(errs)) >= 4.5


# }}}


# {{{ torch oracle derivative checks


def test_torch_step_vjp_vs_finite_differences():
    """The stand-in for ``jax.jacfwd`` (``src/pyshocks/timestepping.py:174``):
    <p, J v> from autograd matches a central difference along v."""
    torch.manual_seed(0)
    n = 64
    rng = np.random.default_rng(3)
    grid = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
    u = torch.tensor(R.random_fourier_ic(rng, grid.f)[3:-3])[None]
    p = torch.randn(1, n, dtype=torch.float64)
    v = torch.randn(1, n, dtype=torch.float64)
    dt = float(T.predict_dt(u, 2.0 / n)[0])
    g = T.step_vjp(u, p, dt, 2.0 / n)
    h = 1.0e-6
    fp = T.ssprk33(u + h * v, dt, 2.0 / n)
    fm = T.ssprk33(u - h * v, dt, 2.0 / n)
    fd = torch.sum(p * (fp - fm)) / (2 * h)
    assert abs(float(torch.sum(g * v) - fd)) < 1.0e-7 * max(1.0, abs(float(fd)))


# }}}


# {{{ Dirichlet / Neumann boundaries (golden runs of the reference)


def dirichlet_data(t, x):
    return 0.6 + 0.25 * np.sin(np.pi * x - t)


def neumann_left(t):
    return 0.3 * np.cos(2.0 * t)


def neumann_right(t):
    return -0.2


BC_RUNS = [
    ("dirichlet_rusanov_n128", "rusanov", "wenojs53", "dirichlet"),
    ("neumann_rusanov_n128", "rusanov", "wenojs53", "neumann"),
    ("dirichlet_eo_wenojs32_n100", "eo", "wenojs32", "dirichlet"),
    ("neumann_godunov_constant_n90", "godunov", "constant", "neumann"),
]


@pytest.mark.parametrize(("name", "flux_kind", "rec", "kind"), BC_RUNS)
def test_numpy_oracle_boundary_runs_golden(name, flux_kind, rec, kind):
    """``apply_boundary`` of ``DirichletBoundary`` / ``NeumannBoundary``
    (``src/pyshocks/scalar.py:397-511``) restated: bit-identical 60-step runs."""
    g = _load(name)
    n = int(g["n"])
    grid = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
    spec = R.SchemeSpec(flux_kind=flux_kind, rec=rec, eps=1.0e-6)
    if kind == "dirichlet":
        def bc(t, u):
            return R.apply_boundary_dirichlet(u, grid, t, dirichlet_data, dirichlet_data)
    else:
        def bc(t, u):
            return R.apply_boundary_neumann(u, grid, t, neumann_left, neumann_right)
    rhs0 = R.apply_operator(spec, grid, g["u0"], 0.0, bc)
    np.testing.assert_array_equal(rhs0, g["rhs0"])  # ghost cells included
    u, dts = R.evolve(spec, grid, g["u0"], theta=1.0, maxit=60, bc=bc)
    np.testing.assert_array_equal(np.array(dts), g["dts"])
    np.testing.assert_array_equal(u, g["u"])


# }}}


# {{{ MUSCL / MUSCLS (golden runs of the reference, reconstruction.py:172-296)


def _muscl_runs():
    out = []
    for p in sorted(GOLDEN.glob("muscl*_n*_s*.npz")):
        parts = p.stem.split("_")
        kind, flux_kind, lim = parts[0], parts[1], parts[2]
        param = 1.0
        if lim in ("minmod", "vanalbada"):
            param = float(parts[3])
        out.append((p.stem, kind, flux_kind, lim, param))
    return out


MUSCL_RUNS = _muscl_runs()


def muscl_spec(kind, flux_kind, lim, param, grid):
    return R.SchemeSpec(flux_kind=flux_kind, rec=kind, limiter=lim, limiter_param=param,
                        atol=1.0e-12, x=grid.x, dx=grid.dx)


@pytest.mark.parametrize(("name", "kind", "flux_kind", "lim", "param"), MUSCL_RUNS)
def test_numpy_oracle_muscl_runs_golden(name, kind, flux_kind, lim, param):
    """The limiters and both MUSCL forms restated: bit-identical 40-step runs."""
    g = _load(name)
    n = int(g["n"])
    grid = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
    spec = muscl_spec(kind, flux_kind, lim, param, grid)
    np.testing.assert_array_equal(R.apply_operator(spec, grid, g["u0"])[3:-3], g["rhs0"][3:-3])
    u, dts = R.evolve(spec, grid, g["u0"], theta=1.0, maxit=40)
    np.testing.assert_array_equal(np.array(dts), g["dts"])
    np.testing.assert_array_equal(u[3:-3], g["u"][3:-3])


@pytest.mark.parametrize(("lim", "param"), [("minmod", 1.0), ("minmod", 1.5), ("minmod", 2.0),
                                            ("mc", 1.0), ("superbee", 1.0), ("vanalbada", 1),
                                            ("vanalbada", 2), ("vanleer", 1.0), ("koren", 1.0)])
@pytest.mark.parametrize("smooth", [True, False])
def test_flux_limiters(lim, param, smooth):
    """``tests/test_muscl.py:38-90``: on a sine the limiter is active somewhere;
    on a step (piecewise constant) it vanishes, i.e. first order everywhere."""
    n = 128
    grid = R.make_uniform_cell_grid(-1.0, 1.0, n, 1)
    if smooth:
        u = np.sin(np.pi * grid.x)
    else:
        u = ((grid.x > -0.5) & (grid.x < 0.5)).astype(np.float64)
    phi = np.pad(R.limiter_phi(lim, R.local_slope_ratio(u), param), 1)
    if smooth:
        assert np.max(phi[1:-1]) > 0.0
    else:
        assert np.max(phi[1:-1]) < 1.0e-12


# }}}


# {{{ the ghosted torch restatement (adjoint_step's oracle) against the NumPy oracle

GHOSTED = [(rec, fk, alpha, kind, g)
           for rec, g in (("constant", 1), ("constant", 3), ("wenojs53", 3))
           for fk, alpha in (("rusanov", 1.0), ("rusanov", 0.98), ("lf", 1.0), ("lf", 0.995))
           for kind in ("periodic", "dirichlet", "neumann")]


def _ghosted_case(rec, fk, alpha, kind, g, n=40, seed=3):
    rng = np.random.default_rng(seed)
    grid = R.make_uniform_cell_grid(-1.0, 1.0, n, g)
    dt = 0.4 * grid.dx_min
    u = R.random_fourier_ic(rng, grid.f)
    spec = R.SchemeSpec(flux_kind=fk, rec=rec, eps=1.0e-6, alpha=alpha)
    data = rng.uniform(-1.0, 1.0, size=(3, 2, 3))
    neu = rng.uniform(-1.0, 1.0, size=(3, 2))
    tb = {"left": kind, "right": kind, "dirichlet": data, "neumann": neu}
    times = (0.0, dt, 0.5 * dt)  # SSPRK33's stage times from t = 0

    def bc(t, v):
        s_ = times.index(t)
        if kind == "periodic":
            return R.apply_boundary_periodic(v, g)
        if kind == "dirichlet":
            return R.apply_boundary_dirichlet(
                v, grid, t, lambda tt, x: data[s_, 0, :g][::-1][: x.size],
                lambda tt, x: data[s_, 1, :g][: x.size])
        return R.apply_boundary_neumann(v, grid, t, lambda tt: neu[s_, 0], lambda tt: neu[s_, 1])

    return grid, u, spec, tb, bc, times, dt


@pytest.mark.parametrize(("rec", "fk", "alpha", "kind", "g"), GHOSTED)
def test_torch_ghosted_operator_and_step_match_numpy_oracle(rec, fk, alpha, kind, g):
    """The ghosted restatement used for the single-instance adjoint oracle
    equals the NumPy oracle on every cell, ghosts included: the operator at
    the first stage time, and one SSPRK33 step with the boundary at the three
    stage times (1e-13 relative)."""
    grid, u, spec, tb, bc, times, dt = _ghosted_case(rec, fk, alpha, kind, g)
    nu = 1.0 if alpha == 1.0 else grid.dx_min ** (alpha - 1)
    kw = dict(rec=rec, flux_kind=fk, eps=1.0e-6, nu=nu)
    x = torch.tensor(grid.x)
    ref = R.apply_operator(spec, grid, u, times[0], bc)
    got = T.ghosted_operator(torch.tensor(u), grid.dx_min, g, tb, 0, x, **kw).numpy()
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(got - ref)) <= 1.0e-13 * scale
    ref = R.ssprk33(lambda t, v: R.apply_operator(spec, grid, v, t, bc), dt, times[0], u)
    got = T.ghosted_advance(torch.tensor(u), dt, grid.dx_min, g, tb, x, **kw).numpy()
    assert np.max(np.abs(got - ref)) <= 1.0e-13 * np.max(np.abs(ref))

# }}}
