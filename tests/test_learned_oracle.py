"""CPU checks of the learned-weight oracle (``oracle/learned_ref.py``): the
left-face rule is WENO-JS5's own structure, and the trust-band fallback is the
reference's WENO-JS5 reconstruction (pinned through ``oracle/numpy_ref.py``,
which the golden vectors pin)."""

from __future__ import annotations

import numpy as np
import torch

from oracle import learned_ref as LR
from oracle import numpy_ref as R


def _stencils(n, seed):
    g = torch.Generator().manual_seed(seed)
    x = torch.linspace(-2, 2, 5, dtype=torch.float64)
    a, b, c = (torch.randn(n, 1, generator=g, dtype=torch.float64) for _ in range(3))
    smooth = a + b * x + 0.3 * c * x**2
    jump = torch.where(x[None, :] > torch.randint(-2, 3, (n, 1), generator=g), 1.0, 0.0)
    return smooth + jump * torch.randn(n, 1, generator=g, dtype=torch.float64)


def test_left_face_is_the_mirror_rule():
    """omega_L = softmax(z2 - ln 3, z1, z0 + ln 3): for JS logits
    z = ln d - 2 ln(eps + beta) this gives the JS weights of the mirrored
    stencil, i.e. the reference's left-face weights."""
    s = _stencils(257, 9)
    jr, jl = LR.js_weights(s, 1.0e-6)
    z = torch.log(jr)
    ln3 = torch.log(torch.tensor(3.0, dtype=z.dtype))
    zl = torch.stack([z[:, 2] - ln3, z[:, 1], z[:, 0] + ln3], dim=-1)
    torch.testing.assert_close(torch.softmax(zl, dim=-1), jl, rtol=1e-12, atol=1e-14)
    jr_m, _ = LR.js_weights(torch.flip(s, dims=(-1,)), 1.0e-6)
    torch.testing.assert_close(jl, jr_m, rtol=1e-12, atol=1e-14)


def test_full_fallback_is_the_reference_wenojs5():
    """band < 0 sends every face to the fallback: the learned reconstruction
    then equals WENO-JS5 (reconstruction.py:358-377) on a periodic row."""
    n, eps = 64, 1.0e-6
    rng = np.random.default_rng(2)
    u = np.cumsum(rng.normal(size=n)) * 0.1
    u[n // 2:] += 1.0
    wts = {"params": LR.init_params(seed=1, dtype=torch.float64), "tau": 1e-2, "band": -1.0,
           "dev": 0.5}
    ul, ur = LR.learned_recon(torch.tensor(u)[None], wts, eps)
    g = 3
    ue = np.concatenate([u[-g:], u, u[:g]])
    rl, rr = R.reconstruct_wenojs(R.weno_js_53_coefficients(), eps, ue)
    np.testing.assert_allclose(ul[0].numpy(), rl[g:-g], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(ur[0].numpy(), rr[g:-g], rtol=1e-12, atol=1e-12)


def test_training_loss_gradient_is_finite_and_pulls_to_ideal():
    """With reg > 0 and targets equal to the ideal-weight face values the
    untrained network (softmax at the ideal weights) is a stationary point."""
    s = _stencils(64, 3)
    p = LR.init_params(seed=0, dtype=torch.float64)
    W1, b1, W2, b2, W3, b3 = LR.unpack(p)
    with torch.no_grad():
        W3.zero_()  # logits = b3 = ln d exactly
    wr, wl = LR.mlp_weights(p, s)
    d = torch.tensor([0.1, 0.6, 0.3], dtype=torch.float64)
    torch.testing.assert_close(wr, d.expand_as(wr))
    torch.testing.assert_close(wl, d.expand_as(wl))
    hr, hl = LR.substencils(s)
    t = torch.stack([(hr * d).sum(-1), (hl * d).sum(-1)], dim=-1)
    pp = p.clone().requires_grad_(True)
    loss = LR.training_loss(pp, s, t, torch.ones(64, dtype=torch.float64), reg=0.5)
    (g,) = torch.autograd.grad(loss, pp)
    assert float(loss.detach()) < 1e-28 and float(g.abs().max()) < 1e-12


def test_library_and_oracle_share_the_trust_band_defaults():
    """The library's LearnedWENO trust-band defaults (tau, band, dev) and
    normalisation floor are the oracle's, so tests that leave them out compare
    the same scheme."""
    import dataclasses
    import inspect

    from pyshocks_gb300 import learned

    lib = {f.name: f.default for f in dataclasses.fields(learned.LearnedWENO)
           if f.name in ("tau", "band", "dev", "norm_eps")}
    sig = inspect.signature(LR.cell_face_values).parameters
    assert lib["dev"] == sig["dev"].default == 0.8
    assert lib["norm_eps"] == sig["norm_eps"].default == LR.NORM_EPS == learned.NORM_EPS
    assert (lib["tau"], lib["band"]) == (1.0e-2, 0.1)
