"""Parity of the batched plain workload at its own scale.

The benchmark's batch (B=4096 Burgers instances, N drawn from {1024, 2048,
4096, 8192, 16384}, 8-mode Fourier + step-jump initial states, WENO-JS5 with
eps 1e-6, Rusanov, SSPRK33, CFL 0.5, 2000 fixed-count steps, float64) is run
for its first 24 instances, which cover all five sizes, with the launch shape
the autotuner picks for the full batch (tile 1024, 3 CTAs/SM) and with the
library default, and compared with the C restatement of the reference path
(``oracle/shocks_ref.c``, which follows ``src/pyshocks/timestepping.py:89-152,
312-320`` and the WENO/Rusanov lines it cites) on every instance.

Tolerances: 1e-10 max-abs on the state after 2000 steps (the stated parity bar
for the float64 path) and 1e-13 relative on every step's dt. The NumPy and C
restatements, whose summation orders differ, agree to 2e-13 and 5e-15 on these
instances, so the bar has three orders of magnitude of headroom.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NSTEPS = 2000
NINST = 24


@pytest.fixture(scope="module")
def workload():
    import bench
    from oracle import c_ref

    sizes, params = bench.workload_params(bench.SEED)
    sizes = sizes[:NINST]
    assert set(int(n) for n in sizes) == set(bench.SIZES)
    u0 = bench.initial_state(sizes, params[:NINST], "cpu").numpy()
    off = np.zeros(NINST + 1, dtype=np.int64)
    off[1:] = np.cumsum(sizes)
    dx = 2.0 / sizes.astype(np.float64)
    ref, dts, _ = c_ref.run_batch(u0, off, dx, theta=bench.THETA, eps=bench.EPS, nsteps=NSTEPS,
                                  want_dts=True)
    return sizes, dx, off, u0, ref, dts


@pytest.mark.parametrize(("tile", "ctas"), [(1024, 3), (0, 0)])
def test_workload_2000_steps_match_oracle(workload, tile, ctas):
    import bench
    import pyshocks_gb300 as gb
    from pyshocks_gb300.batched import BatchedSolver

    sizes, dx, off, u0, ref, dts = workload
    rec = gb.reconstruction.make_reconstruction_from_name("wenojs53", eps=bench.EPS)
    scheme = gb.burgers.make_scheme_from_name("rusanov", rec=rec)
    solver = BatchedSolver(scheme, sizes, dx, theta=bench.THETA, tile=tile, ctas_per_sm=ctas,
                           max_steps=NSTEPS)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        solver.reset(torch.tensor(u0))
        solver.step(NSTEPS, graph=True)
        u = solver.u.cpu().numpy()
        hist = solver.dt_history().cpu().numpy()
    stream.synchronize()
    assert solver.status() == 0
    assert hist.shape == (NSTEPS, NINST)
    for b, n in enumerate(sizes):
        err = np.max(np.abs(u[off[b]:off[b + 1]] - ref[off[b]:off[b + 1]]))
        assert err <= 1.0e-10, (b, int(n), err)
    rel = np.max(np.abs(hist - dts) / dts)
    assert rel <= 1.0e-13, rel
