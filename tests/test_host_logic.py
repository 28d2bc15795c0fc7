"""Host-side logic that needs no GPU: boundary tables, the autotuner's
candidate shapes and shared-memory estimates, packing and the instance
partition."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from pyshocks_gb300 import _lib as L
from pyshocks_gb300 import autotune
from pyshocks_gb300.batched import _boundary_tables, pack_offsets, partition_instances


def test_boundary_tables_broadcast_and_kinds():
    lk, rk, d, nm = _boundary_tables(3, torch.device("cpu"), "dirichlet", None, [0.5, -0.25], None)
    assert (lk, rk) == (L.SHK_BC_DIRICHLET, L.SHK_BC_DIRICHLET)
    assert d.shape == (3, 2, 3) and d.dtype == torch.float64 and nm is None
    assert torch.all(d[:, 0, :] == 0.5) and torch.all(d[:, 1, :] == -0.25)
    full = np.arange(12.0).reshape(2, 2, 3)
    _, _, d2, _ = _boundary_tables(2, torch.device("cpu"), "dirichlet", "neumann", full,
                                   [[1.0, 2.0], [3.0, 4.0]])
    assert torch.equal(d2, torch.tensor(full))
    lk, rk, d, nm = _boundary_tables(4, torch.device("cpu"), "neumann", None, None, [0.0, 1.0])
    assert (lk, rk) == (L.SHK_BC_NEUMANN, L.SHK_BC_NEUMANN)
    assert nm.shape == (4, 2) and torch.all(nm[:, 1] == 1.0)
    with pytest.raises(KeyError):
        _boundary_tables(1, torch.device("cpu"), "reflecting", None, None, None)


def test_autotune_candidates_fit_shared_memory():
    smem = autotune.SMEM_PER_SM
    for dtype in (torch.float64, torch.float32):
        for learned in (False, True):
            for adjoint in (False, True):
                weno5 = not learned
                cands = autotune.candidates(dtype, 16384, learned, adjoint, weno5)
                assert cands, (dtype, learned, adjoint)
                for tile, cps in cands:
                    per = autotune._smem_bytes(tile, dtype, learned, weno5)
                    assert per <= smem and (cps == 0 or cps * per <= smem)
                    if adjoint:
                        assert autotune._adjoint_smem_bytes(tile, dtype, learned) <= smem
    # short instances: no tile longer than twice the largest instance (but 512 stays)
    assert all(t <= 512 for t, _ in autotune.candidates(torch.float64, 100))
    # the float WENO-JS5 step's 6-array layout admits 4 CTAs of tile 2048
    assert (2048, 4) in autotune.candidates(torch.float32, 16384, weno5=True)


def test_pack_offsets_and_partition():
    sizes = [5, 1024, 3, 77, 2048, 96]
    off = pack_offsets(sizes)
    assert off[0] == 0 and np.all(np.diff(off) == sizes)
    parts = partition_instances(sizes, 3)
    assert sorted(np.concatenate(parts).tolist()) == list(range(len(sizes)))
    loads = [sum(sizes[i] for i in p) for p in parts]
    assert max(loads) == 2048  # LPT: the largest instance alone bounds the makespan


def test_bench_workload_is_the_batched_configuration():
    """The bench's synthetic batch: 4096 instances with N from {1024, ..., 16384}
    (25,865,216 cells for the committed seed), and initial states that are the
    exact cell averages of m + sum_k A_k sin(k pi x + phi_k) plus 0-3 steps,
    checked against an independent per-cell quadrature (Gauss-Legendre for the
    smooth part, the covered fraction of the cell for each step)."""
    import importlib.util
    import pathlib

    spec = importlib.util.spec_from_file_location(
        "bench_for_test", pathlib.Path(__file__).resolve().parents[1] / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)

    sizes, params = bench.workload_params(bench.SEED)
    assert sizes.size == 4096 and set(np.unique(sizes)) <= set(bench.SIZES)
    assert int(sizes.sum()) == 25_865_216
    assert all(-0.5 <= p[0] <= 0.5 and 0 <= len(p[3]) <= 3 for p in params)

    pick = [0, 1, 2]
    sub_sizes = sizes[pick]
    u = bench.initial_state(sub_sizes, [params[i] for i in pick], "cpu").numpy()
    xi, wi = np.polynomial.legendre.leggauss(8)
    at = 0
    for b, n in zip(pick, sub_sizes):
        m, amp, phi, hj, xj = params[b]
        h = 2.0 / n
        f = -1.0 + h * np.arange(n + 1)
        xm = 0.5 * (f[1:] + f[:-1])
        xq = xm[:, None] + 0.5 * h * xi[None, :]
        smooth = m + sum(a * np.sin((k + 1) * np.pi * xq + p) for k, (a, p) in enumerate(zip(amp, phi)))
        ref = (smooth * wi[None, :]).sum(1) * 0.5
        for hh, x0 in zip(hj, xj):
            ref += hh * np.clip((f[1:] - x0) / h, 0.0, 1.0)
        assert np.max(np.abs(u[at:at + n] - ref)) < 1.0e-11, b
        at += n


def test_timestep_helpers_follow_the_reference():
    """``predict_timestep_from_resolutions`` / ``predict_maxit_from_timestep`` /
    ``predict_timestep_from_maxit`` (``src/pyshocks/timestepping.py:242-280``)."""
    from pyshocks_gb300 import timestepping as ts

    dt = ts.predict_timestep_from_resolutions(-1.0, 1.0, [64, 128, 96], umax=10.0)
    assert dt == (2.0 / 128) / 10.0
    assert ts.predict_timestep_from_resolutions(0.0, 1.0, [10], p=2) == 0.1**2
    maxit, dt2 = ts.predict_maxit_from_timestep(1.0, dt)
    assert maxit == int(1.0 / dt) and dt2 == 1.0 / maxit + 1.0e-15
    assert ts.predict_timestep_from_maxit(2.0, 8) == (8, 0.25 + 1.0e-15)


def test_scheme_names_follow_the_reference():
    """The reference's Burgers scheme names (``src/pyshocks/burgers/__init__.py:62-98``):
    the finite-volume ones build, the summation-by-parts ones say they are not
    on this path, unknown names raise ValueError."""
    from pyshocks_gb300 import burgers, reconstruction

    weno = reconstruction.WENOJS53()
    for name in ("default", "godunov", "rusanov", "lf", "eo"):
        assert burgers.make_scheme_from_name(name, rec=weno).rec is weno
    assert burgers.make_scheme_from_name("esweno32", rec=reconstruction.ESWENO32()) is not None
    assert type(burgers.make_scheme_from_name("default", rec=weno)).__name__ == "LaxFriedrichs"
    for name in ("ssmuscl", "ssweno242", "splitrusanov"):
        with pytest.raises(NotImplementedError):
            burgers.make_scheme_from_name(name)
    with pytest.raises(ValueError):
        burgers.make_scheme_from_name("nope")
    # reconstructions (src/pyshocks/reconstruction.py:528-566)
    for name in ("default", "constant", "muscl", "muscls", "wenojs32", "wenojs53", "esweno32"):
        assert reconstruction.make_reconstruction_from_name(name) is not None
    with pytest.raises(NotImplementedError):
        reconstruction.make_reconstruction_from_name("ssweno242")


@pytest.mark.parametrize(("bits", "exc", "match"), [
    (0, None, None),
    (L.ERR_NONFINITE, ValueError, "not finite"),
    (L.ERR_TIMEOUT, RuntimeError, "bounded device wait"),
    (L.ERR_BOUNDS, RuntimeError, "left its array"),
    (L.ERR_NONFINITE | L.ERR_TIMEOUT, ValueError, "not finite"),
])
def test_status_bits_raise_on_the_host(bits, exc, match):
    """BatchedSolver.check_status decodes the plan's status word: the device
    sets ERR_NONFINITE (the reference's non-finite dt ValueError,
    timestepping.py:144-145), ERR_TIMEOUT (an expired bounded wait) or
    ERR_BOUNDS (the bounds-check build); the word is read through status(),
    replaced here by a stub returning the bits."""
    from pyshocks_gb300.batched import BatchedSolver

    s = object.__new__(BatchedSolver)
    s.status = lambda: bits
    if exc is None:
        s.check_status()
    else:
        with pytest.raises(exc, match=match):
            s.check_status()
