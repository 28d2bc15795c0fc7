"""The Lax-Friedrichs operator entry point that allocates nothing.

Callers such as a JAX custom-call handler cannot allocate device memory of
their own: JAX holds most of the GPU in its own pool and passes the handler
only the operand buffers. ``shk_apply_operator_lf_noalloc_f64`` serves them
by keeping its scratch in a fixed array inside ``libshocks.so``. These checks
call it through the C ABI and compare it with the regular path
(``shk_max_wavespeed_f64`` + ``shk_apply_operator_f64``, which uses a
caller-allocated scratch value) on two calls in a row, to the 1e-12 relative
tolerance of the other operator tests. The file is named so pytest collects it
last; it passes on its own in a fresh process as well.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import numpy_ref as R

pytestmark = pytest.mark.gpu


def _scheme(L):
    # Lax-Friedrichs + WENO-JS5, Burgers (reconstruction.py:335-348, burgers/schemes.py:136-153)
    return L.ShkScheme(flux=L.SHK_FLUX_LF, rec=L.SHK_REC_WENOJS53, equation=L.SHK_EQ_BURGERS,
                       eps=1.0e-6, delta=0.0, nu=1.0, speed=1.0)


def _ghosted_state(n, seed):
    og = R.make_uniform_cell_grid(-1.0, 1.0, n, 3)
    u0 = R.random_fourier_ic(np.random.default_rng(seed), og.f)
    return torch.tensor(u0, device="cuda"), og


def _regular(L, lib, s, u, n, dx, stream):
    amax = torch.empty((), dtype=torch.float64, device="cuda")
    out = torch.empty_like(u)
    L.check(lib.shk_max_wavespeed_f64(s, u.data_ptr(), n, 3, amax.data_ptr(), stream))
    L.check(lib.shk_apply_operator_f64(s, u.data_ptr(), out.data_ptr(), n, 3, dx,
                                       amax.data_ptr(), stream))
    return out


def test_noalloc_matches_regular_path_twice():
    from pyshocks_gb300 import _lib as L

    lib = L.lib()
    s = _scheme(L)
    stream = L.stream_handle()
    # the first call is larger than the second: stale partial maxima left in
    # the shared scratch by call 1 must not leak into call 2
    for n, seed in [(70001, 1), (3000, 2)]:
        u, og = _ghosted_state(n, seed)
        dx = 2.0 / n
        out = torch.empty_like(u)
        st = lib.shk_apply_operator_lf_noalloc_f64(s, u.data_ptr(), out.data_ptr(), n, 3, dx,
                                                   stream)
        assert st == L.SHK_OK, L.errstr(st)
        ref = _regular(L, lib, s, u, n, dx, stream)
        torch.cuda.synchronize()
        a = out[3:-3].cpu().numpy()
        b = ref[3:-3].cpu().numpy()
        scale = np.max(np.abs(b))
        assert np.max(np.abs(a - b)) / scale < 1.0e-12
        # and both agree with the oracle's global Lax-Friedrichs operator
        o = R.apply_operator(R.SchemeSpec(flux_kind="lf"), og, u.cpu().numpy())[3:-3]
        assert np.max(np.abs(a - o)) / scale < 1.0e-12


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from pyshocks_gb300 import _lib as L

    lib = L.lib()
    limit = lib.shk_apply_operator_lf_noalloc_max_cells()
    assert limit == 4096 * 512
    u = torch.zeros(16, dtype=torch.float64, device="cuda")
    # rejected on the host before any launch, so the small buffer is never read
    st = lib.shk_apply_operator_lf_noalloc_f64(_scheme(L), u.data_ptr(), u.data_ptr(),
                                               limit + 1, 3, 1.0e-3, L.stream_handle())
    assert st == L.SHK_ETOOLARGE
