"""Generate the golden vectors under ``tests/golden/`` by running the reference's
own Python source (alexfikl/pyshocks, ``src/pyshocks``) unmodified.

JAX is not installed in the build container, so the reference is imported on
top of ``tests/golden/jaxshim`` -- a small NumPy-backed stand-in for the
``jax`` / ``jax.numpy`` calls on the forward path. The arithmetic executed is
the reference's (its stencils, its operation order, its ``step`` loop); only
the array runtime underneath differs (NumPy instead of XLA, so sums inside
``jnp.convolve`` follow NumPy's order).

Usage (needs the reference checkout; writes ``tests/golden/*.npz``)::

    python tests/golden/make_golden.py /path/to/pyshocks

The fixtures are committed; the tests read them without the reference.
"""

from __future__ import annotations

import importlib.metadata as _md
import pathlib
import sys
from dataclasses import dataclass

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]


def _import_reference(refdir: pathlib.Path):
    sys.path.insert(0, str(HERE / "jaxshim"))
    sys.path.insert(0, str(refdir / "src"))
    sys.path.insert(0, str(REPO))
    orig = _md.version
    _md.version = lambda name: "0+numpy-shim" if name == "pyshocks" else orig(name)
    import pyshocks  # noqa: F401

    return pyshocks


def main(refdir: pathlib.Path) -> None:
    _import_reference(refdir)
    import jax.numpy as jnp
    from pyshocks import (
        ConservationLawScheme,
        apply_operator,
        bind,
        burgers,
        flux,
        make_uniform_cell_grid,
        numerical_flux,
        predict_timestep,
        reconstruction,
        timestepping,
        weno,
    )
    from pyshocks.scalar import PeriodicBoundary, scalar_flux_rusanov

    from oracle import numpy_ref as R  # inputs only (initial conditions)

    out: dict[str, dict[str, np.ndarray]] = {}

    # {{{ reconstruction kernels on fixed data (tests/test_weno.py:34-166 inputs)

    for name, is_smooth in [("sine", True), ("step", False)]:
        n = 64 + 4
        theta = np.linspace(0.0, 2.0 * np.pi, n)
        u = np.sin(theta) if is_smooth else (theta < np.pi).astype(np.float64)
        uj = jnp.array(u)
        case = {"u": u}
        for rname, kw in [("wenojs53", {"eps": 1.0e-6}), ("wenojs32", {"eps": 1.0e-6}),
                          ("esweno32", {"eps": 1.0e-6, "delta": 1.0e-6})]:
            rec = reconstruction.make_reconstruction_from_name(rname, **kw)
            case[f"{rname}_beta"] = np.asarray(weno.weno_smoothness(rec.s, uj))
            case[f"{rname}_uhat"] = np.asarray(weno.weno_interp(rec.s, uj))
            if rname == "esweno32":
                case[f"{rname}_omega"] = np.asarray(weno.es_weno_weights(rec.s, uj, eps=rec.eps))
            else:
                case[f"{rname}_omega"] = np.asarray(weno.weno_js_weights(rec.s, uj, eps=rec.eps))
            grid = make_uniform_cell_grid(-1.0, 1.0, n - 2 * rec.stencil_width,
                                          nghosts=rec.stencil_width)
            ul, ur = reconstruction.reconstruct(rec, grid, None, uj, uj, uj)
            case[f"{rname}_ul"] = np.asarray(ul)
            case[f"{rname}_ur"] = np.asarray(ur)
        out[f"recon_{name}"] = case

    # }}}

    # {{{ schemes

    @dataclass(frozen=True)
    class LWRRusanov(burgers.Rusanov):
        """LWR traffic flux rho (1 - rho) plugged in through the reference's
        singledispatch API (pattern of examples/traffic-flow-model.py:14-39)."""

    @flux.register(LWRRusanov)
    def _flux_lwr(scheme, t, x, u):
        return (1 - u) * u

    @numerical_flux.register(LWRRusanov)
    def _nflux_lwr(scheme, grid, bc, t, u):
        return scalar_flux_rusanov(scheme, grid, bc.boundary_type, t, 1 - 2 * u, u,
                                   alpha=scheme.alpha)

    @predict_timestep.register(LWRRusanov)
    def _dt_lwr(scheme, grid, bc, t, u):
        smax = jnp.max(jnp.abs(1 - 2 * u[grid.i_]))
        return 0.5 * grid.dx_min / smax

    def make_scheme(kind: str):
        if kind == "rusanov":
            rec = reconstruction.make_reconstruction_from_name("wenojs53", eps=1.0e-6)
            return burgers.make_scheme_from_name("rusanov", rec=rec)
        if kind == "lf":
            rec = reconstruction.make_reconstruction_from_name("wenojs53", eps=1.0e-6)
            return burgers.make_scheme_from_name("lf", rec=rec)
        if kind == "esweno":
            rec = reconstruction.make_reconstruction_from_name("esweno32")
            return burgers.make_scheme_from_name("esweno32", rec=rec)
        if kind == "lwr":
            rec = reconstruction.make_reconstruction_from_name("wenojs53", eps=1.0e-6)
            return LWRRusanov(rec=rec)
        # "<scheme>-<reconstruction>": the other Burgers fluxes and reconstructions;
        # "<scheme>-muscl[s]_<limiter>[_<param>]": MUSCL with a limiter
        sname, rname = kind.split("-")
        if rname.startswith("muscl"):
            from pyshocks.limiters import make_limiter_from_name

            parts = rname.split("_")
            lkw = {}
            if parts[1] == "minmod":
                lkw["theta"] = float(parts[2])
            elif parts[1] == "vanalbada":
                lkw["variant"] = int(parts[2])
            lm = make_limiter_from_name(parts[1], **lkw)
            cls = reconstruction.MUSCLS if parts[0] == "muscls" else reconstruction.MUSCL
            return burgers.make_scheme_from_name(sname, rec=cls(lm=lm))
        rec = reconstruction.make_reconstruction_from_name(rname, eps=1.0e-6)
        return burgers.make_scheme_from_name(sname, rec=rec)

    bc = PeriodicBoundary()

    def run(kind, n, u0_fn, *, tfinal=None, maxit=None, theta=1.0, bc=bc):
        scheme = make_scheme(kind)
        grid = make_uniform_cell_grid(-1.0, 1.0, n, nghosts=3)
        scheme = bind(scheme, grid, bc)
        u0 = u0_fn(grid)
        method = timestepping.SSPRK33(
            predict_timestep=lambda t, u: theta * predict_timestep(scheme, grid, bc, t, u),
            source=lambda t, u: apply_operator(scheme, grid, bc, t, u),
            checkpoint=None,
        )
        dts = []
        for ev in timestepping.step(method, jnp.array(u0), tfinal=tfinal, maxit=maxit):
            if ev.iteration > 0:
                dts.append(float(ev.dt))
        res = {
            "u0": np.asarray(u0),
            "u": np.asarray(ev.u),
            "dts": np.array(dts),
            "t": np.array(float(ev.t)),
            "n": np.array(n),
            "rhs0": np.asarray(apply_operator(scheme, grid, bc, 0.0, jnp.array(u0))),
            "dt0": np.array(float(theta * predict_timestep(scheme, grid, bc, 0.0, jnp.array(u0)))),
        }
        if kind == "esweno":
            res["eps"] = np.array(float(scheme.rec.eps))
            res["delta"] = np.array(float(scheme.rec.delta))
        return res

    def sine_ic(grid):
        og = R.make_uniform_cell_grid(-1.0, 1.0, int(grid.x.size) - 6, 3)
        return R.exact_cell_average_sine(og)

    def fourier_ic(seed):
        def fn(grid):
            rng = np.random.default_rng(seed)
            return R.random_fourier_ic(rng, np.asarray(grid.f))

        return fn

    def lwr_ic(seed):
        def fn(grid):
            rng = np.random.default_rng(seed)
            return R.lwr_ic(rng, np.asarray(grid.f))

        return fn

    # the parity workload: N = 256, t_final = 1, CFL 0.5
    out["sine_rusanov_n256"] = run("rusanov", 256, sine_ic, tfinal=1.0)
    out["sine_lf_n256"] = run("lf", 256, sine_ic, tfinal=1.0)
    out["sine_esweno_n256"] = run("esweno", 256, sine_ic, tfinal=1.0)
    # short fixed-count runs on random data (the batched workload's generator)
    for seed, n in [(11, 64), (12, 96), (13, 128), (14, 50)]:
        out[f"fourier_rusanov_n{n}_s{seed}"] = run("rusanov", n, fourier_ic(seed), maxit=40)
    out["fourier_lf_n64_s21"] = run("lf", 64, fourier_ic(21), maxit=40)
    out["fourier_esweno_n64_s22"] = run("esweno", 64, fourier_ic(22), maxit=40)
    out["lwr_rusanov_n128_s31"] = run("lwr", 128, lwr_ic(31), maxit=60)
    # Dirichlet and Neumann boundaries (scalar.py:397-511) with time-dependent
    # data: g_d(t, x) = 0.6 + 0.25 sin(pi x - t), g_n(t) = 0.3 cos(2 t) on the
    # left, -0.2 on the right
    from pyshocks.scalar import make_dirichlet_boundary, make_neumann_boundary

    dbc = make_dirichlet_boundary(ga=lambda t, x: 0.6 + 0.25 * jnp.sin(jnp.pi * x - t))
    nbc = make_neumann_boundary(ga=lambda t: 0.3 * jnp.cos(2.0 * t), gb=lambda t: jnp.array(-0.2))

    def smooth_ic(grid):
        x = np.asarray(grid.x)
        return 0.6 + 0.25 * np.sin(np.pi * x) + 0.1 * np.cos(3.0 * np.pi * x)

    out["dirichlet_rusanov_n128"] = run("rusanov", 128, smooth_ic, maxit=60, bc=dbc)
    out["neumann_rusanov_n128"] = run("rusanov", 128, smooth_ic, maxit=60, bc=nbc)
    out["dirichlet_eo_wenojs32_n100"] = run("eo-wenojs32", 100, smooth_ic, maxit=60, bc=dbc)
    out["neumann_godunov_constant_n90"] = run("godunov-constant", 90, smooth_ic, maxit=60, bc=nbc)

    # MUSCL (flux limiters) and MUSCLS (slope limiters), reconstruction.py:172-296
    for lim in ("none", "minmod_1.0", "minmod_1.5", "mc", "superbee", "vanalbada_1",
                "vanalbada_2", "vanleer", "koren"):
        out[f"muscl_godunov_{lim}_n96_s51"] = run(f"godunov-muscl_{lim}", 96, fourier_ic(51),
                                                  maxit=40)
    for lim in ("minmod_1.0", "mc", "superbee", "vanalbada_1", "vanalbada_2", "vanleer"):
        out[f"muscls_godunov_{lim}_n96_s52"] = run(f"godunov-muscls_{lim}", 96, fourier_ic(52),
                                                   maxit=40)
    out["muscl_rusanov_minmod_1.0_n128_s53"] = run("rusanov-muscl_minmod_1.0", 128,
                                                    fourier_ic(53), maxit=40)
    out["muscls_eo_mc_n128_s54"] = run("eo-muscls_mc", 128, fourier_ic(54), maxit=40)

    # Godunov / Engquist-Osher fluxes and the constant / WENO-JS32 reconstructions
    out["sine_godunov_wenojs53_n256"] = run("godunov-wenojs53", 256, sine_ic, tfinal=1.0)
    out["sine_eo_wenojs53_n256"] = run("eo-wenojs53", 256, sine_ic, tfinal=1.0)
    for sname in ("rusanov", "godunov", "eo"):
        for rname, seed in (("constant", 41), ("wenojs32", 42)):
            out[f"fourier_{sname}_{rname}_n96_s{seed}"] = run(f"{sname}-{rname}", 96,
                                                               fourier_ic(seed), maxit=40)

    # }}}

    for name, case in out.items():
        np.savez_compressed(HERE / f"{name}.npz", **case)
        print(f"wrote {name}.npz ({len(case)} arrays)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of a pyshocks source checkout>")
    main(pathlib.Path(sys.argv[1]))
