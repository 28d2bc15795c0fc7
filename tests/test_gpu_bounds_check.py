"""The kernels under the bounds-check build, and a bounded wait that runs out.

``libshocks_check.so`` is the same sources as ``libshocks.so`` compiled with
``-DSHOCKS_BOUNDS_CHECK``: every index into a window array, the stage storage
or a state array is checked against its array, and a violation is logged
(``shk_check_bounds``) and reported as ``ERR_BOUNDS`` in the plan status
instead of touching memory (``include/shocks_check.h``). With no memory checker
available on the target machines, this build is the memory-safety evidence:

* the oracle-parity tests of the forward, boundary, adjoint, learned and
  no-allocation paths and the tile-independence tests of the plain steps run
  again, with every parameter set they declare and the checked library in
  place of the product one, and must leave the log empty (their own oracle
  tolerances still apply);
* ragged and odd-sized batches (7, 50, 333 and 3001 cells; tiles 64 and 1024;
  float64 and float32) match the oracle with plan status 0;
* the forced-timeout hook makes the loader's bounded wait expire on a tiny plan
  (all copies land, the barrier never completes): the step reports
  ``ERR_TIMEOUT``, ``check_status`` raises, and the same context then steps
  normally again.
"""

from __future__ import annotations

import contextlib
import ctypes
import importlib
import inspect

import numpy as np
import pytest
import torch

from oracle import numpy_ref as R

pytestmark = pytest.mark.gpu

@pytest.fixture(scope="module")
def checked():
    from pyshocks_gb300 import _build
    from pyshocks_gb300 import _lib as L

    if not L.CHECK_LIB_PATH.exists():
        _build.build(variants=("check",))
    return L.load_check_library()


@contextlib.contextmanager
def library(cdll):
    """Route every call of the package through *cdll* (objects created inside
    keep it)."""
    from pyshocks_gb300 import _lib as L

    L.lib()  # the product library is loaded first, as in any other test
    old = L._lib
    L._lib = cdll
    try:
        yield
    finally:
        L._lib = old


def read_log(cdll, reset: bool = True):
    flag, block, thread = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    off, ext = ctypes.c_int64(), ctypes.c_int64()
    st = cdll.shk_check_bounds(1 if reset else 0, ctypes.byref(flag), ctypes.byref(block),
                               ctypes.byref(thread), ctypes.byref(off), ctypes.byref(ext))
    assert st == 0
    return {"flag": flag.value, "block": block.value, "thread": thread.value,
            "offset": off.value, "extent": ext.value}


# {{{ the parity tests, again, under the checked library

RERUN = [
    ("test_gpu_forward", "test_apply_operator_matches_oracle"),
    ("test_gpu_forward", "test_fused_step_matches_oracle"),
    ("test_gpu_forward", "test_batched_uneven_matches_oracle"),
    ("test_gpu_forward", "test_host_stepper_equals_device_plan"),
    ("test_gpu_forward", "test_batched_lax_friedrichs_matches_oracle"),
    ("test_gpu_boundary", "test_apply_operator_with_boundary_matches_oracle"),
    ("test_gpu_boundary", "test_batched_plan_with_boundary_matches_oracle"),
    ("test_gpu_boundary", "test_batched_adjoint_with_boundary_against_finite_differences"),
    ("test_gpu_boundary", "test_single_step_vjp_with_boundary_against_finite_differences"),
    ("test_gpu_boundary", "test_batched_plan_with_time_dependent_dirichlet_matches_oracle"),
    ("test_gpu_adjoint", "test_single_step_vjp_matches_autograd"),
    ("test_gpu_adjoint", "test_batched_checkpointed_gradient_matches_autograd"),
    ("test_gpu_adjoint", "test_stored_stages_and_faces_give_the_same_gradient"),
    ("test_gpu_adjoint", "test_plain_results_do_not_depend_on_the_tile"),
    ("test_gpu_adjoint", "test_float32_lwr_steps_do_not_depend_on_the_tile"),
    ("test_gpu_learned", "test_learned_batched_step_matches_oracle"),
    ("test_gpu_learned", "test_learned_adjoint_matches_autograd"),
    ("test_gpu_learned", "test_stored_stage_states_give_the_same_gradient"),
    ("test_gpu_learned", "test_tensor_core_faces_match_oracle"),
    ("test_gpu_ghosted", "test_ghosted_operator_and_step_match_oracle"),
    ("test_gpu_ghosted", "test_ghosted_vjp_matches_autograd"),
    ("test_zz_no_alloc", "test_noalloc_matches_regular_path_twice"),
]


def _param_sets(fn):
    """Every argument set of *fn*'s ``pytest.mark.parametrize`` marks."""
    sets = [{}]
    for mark in getattr(fn, "pytestmark", []):
        if mark.name != "parametrize":
            continue
        names, values = mark.args[0], mark.args[1]
        names = [s.strip() for s in names.split(",")] if isinstance(names, str) else list(names)
        grown = []
        for s in sets:
            for v in values:
                v = v.values if hasattr(v, "values") else v
                vals = tuple(v) if len(names) > 1 else (v,)
                grown.append({**s, **dict(zip(names, vals))})
        sets = grown
    return sets


def _cases():
    out = []
    for modname, fname in RERUN:
        fn = getattr(importlib.import_module(modname), fname)
        for i, kw in enumerate(_param_sets(fn)):
            out.append(pytest.param(modname, fname, kw, id=f"{fname}-{i}"))
    return out


@pytest.mark.parametrize(("modname", "fname", "kwargs"), _cases())
def test_parity_tests_leave_no_bounds_violation(checked, modname, fname, kwargs):
    import pyshocks_gb300 as gb

    fn = getattr(importlib.import_module(modname), fname)
    kw = dict(kwargs)
    if "gb" in inspect.signature(fn).parameters:
        kw["gb"] = gb
    with library(checked):
        read_log(checked, reset=True)
        fn(**kw)
        log = read_log(checked, reset=True)
    assert log["flag"] == 0, log

# }}}


def _solver_case(sizes, seed):
    u0s = []
    for b, n in enumerate(sizes):
        og = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
        u0s.append(R.random_fourier_ic(np.random.default_rng(seed + b), og.f)[3:-3])
    return u0s


@pytest.mark.parametrize("tile", [64, 1024])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_ragged_batches_match_oracle_under_bounds_check(checked, tile, dtype):
    """Instances shorter than the halo (7), than a tile (50, 333) and odd
    multi-tile ones (3001), 20 fixed-count steps, against the oracle."""
    from pyshocks_gb300 import _lib as L
    from pyshocks_gb300 import burgers, reconstruction
    from pyshocks_gb300.batched import BatchedSolver

    sizes = [7, 50, 333, 3001]
    nsteps = 20
    u0s = _solver_case(sizes, 40)
    refs = []
    for n, u0 in zip(sizes, u0s):
        og = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
        g = np.concatenate([u0[-3:], u0, u0[:3]])
        refs.append(R.evolve(R.SchemeSpec(), og, g, theta=0.8, maxit=nsteps)[0][3:-3])
    rec = reconstruction.make_reconstruction_from_name("wenojs53", eps=1.0e-6)
    with library(checked):
        read_log(checked, reset=True)
        solver = BatchedSolver(burgers.Rusanov(rec=rec), sizes, [2.0 / n for n in sizes],
                               theta=0.8, tile=tile, dtype=dtype, max_steps=nsteps)
        solver.reset(torch.tensor(np.concatenate(u0s)))
        solver.step(nsteps)
        status = solver.status()
        log = read_log(checked, reset=True)
    assert log["flag"] == 0, log
    assert status == 0 and not status & L.ERR_BOUNDS
    tol = 1.0e-11 if dtype == torch.float64 else 2.0e-5
    for b, ref in enumerate(refs):
        u = solver.instance(b).double().cpu().numpy()
        assert np.max(np.abs(u - ref)) / max(1.0, np.max(np.abs(ref))) < tol, (sizes[b], tile)


def test_bounded_wait_runs_out_and_reports_timeout(checked):
    """One aligned instance (N=1024: the loader takes the bulk-copy path). The
    hook makes every wait expect 16 bytes more than its copies deliver and poll
    1024 times: the step kernel records ERR_TIMEOUT and returns; the host
    stepper ORs it from its chunks; check_status raises. With the hook off
    the same plan, in the same context, steps to the oracle's result."""
    from pyshocks_gb300 import _lib as L
    from pyshocks_gb300 import burgers, reconstruction
    from pyshocks_gb300.batched import BatchedSolver, HostStepper

    n = 1024
    u0 = _solver_case([n], 7)[0]
    og = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
    ref = R.evolve(R.SchemeSpec(), og, np.concatenate([u0[-3:], u0, u0[:3]]), theta=1.0,
                   maxit=2)[0][3:-3]
    rec = reconstruction.make_reconstruction_from_name("wenojs53", eps=1.0e-6)
    scheme = burgers.Rusanov(rec=rec)
    with library(checked):
        solver = BatchedSolver(scheme, [n], 2.0 / n, tile=1024)
        hs = HostStepper(scheme, [n, n, n], 2.0 / n, chunks=3)
        host = torch.tensor(np.tile(u0, 3))
        solver.reset(torch.tensor(u0))
        assert checked.shk_check_force_timeout(16, 1024) == 0
        try:
            solver.step(1)
            hs.advance(host, None, 1)
            torch.cuda.synchronize()
            st_plan = solver.status()
            st_host = hs.status()
        finally:
            assert checked.shk_check_force_timeout(0, 0) == 0
        assert st_plan & L.ERR_TIMEOUT, st_plan
        assert st_host & L.ERR_TIMEOUT, st_host
        with pytest.raises(RuntimeError, match="bounded device wait"):
            solver.check_status()
        # the context is usable and the plan steps normally again
        solver.reset(torch.tensor(u0))
        solver.step(2)
        assert solver.status() == 0
        u = solver.u.cpu().numpy()
        log = read_log(checked, reset=True)
    assert log["flag"] == 0, log
    assert np.max(np.abs(u - ref)) < 1.0e-12
