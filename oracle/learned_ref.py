"""torch-CPU restatement of the learned-weight WENO reconstruction.

THIS IS TEST INFRASTRUCTURE (the oracle) for ``pyshocks_gb300/csrc/learned.cu``:
only tests use it, as the checker.

The method (no reference counterpart; it plugs into the reference's
reconstruction slot, ``src/pyshocks/reconstruction.py:79-119``): an MLP
5 -> 32 -> 32 -> 3 (tanh, tanh, softmax) maps the normalised 5-point stencil
of a face to the three nonlinear weights of the WENO-JS5 sub-stencils
(``src/pyshocks/weno.py:206-244``). The face value is the convex combination
``sum_k omega_k uhat_k`` of the sub-stencil values, so the flux stays
conservative. Where the network puts more than ``band`` of its weight on
sub-stencils that WENO-JS marks as crossing a discontinuity (JS weight below
``tau``), or moves any weight more than ``dev`` from the JS weight, the plain
WENO-JS weights are used instead (per face).

Parameter vector (1347 float32): W1[32,5], b1[32], W2[32,32], b2[32],
W3[3,32], b3[3], row-major.
"""

from __future__ import annotations

import torch

N_IN, N_H, N_OUT = 5, 32, 3
N_PARAMS = N_H * N_IN + N_H + N_H * N_H + N_H + N_OUT * N_H + N_OUT
NORM_EPS = 1.0e-12
_D53 = (0.1, 0.6, 0.3)


def unpack(params: torch.Tensor):
    p = params
    i = 0
    W1 = p[i:i + N_H * N_IN].reshape(N_H, N_IN); i += N_H * N_IN
    b1 = p[i:i + N_H]; i += N_H
    W2 = p[i:i + N_H * N_H].reshape(N_H, N_H); i += N_H * N_H
    b2 = p[i:i + N_H]; i += N_H
    W3 = p[i:i + N_OUT * N_H].reshape(N_OUT, N_H); i += N_OUT * N_H
    b3 = p[i:i + N_OUT]; i += N_OUT
    assert i == N_PARAMS
    return W1, b1, W2, b2, W3, b3


def _bf16(x: torch.Tensor, on: bool) -> torch.Tensor:
    return x.to(torch.bfloat16).to(x.dtype) if on else x


def normalise(s: torch.Tensor) -> torch.Tensor:
    """``(s - mean) / (max - min + 1e-12)`` of stencils ``s[..., 5]``."""
    m = s.mean(dim=-1, keepdim=True)
    r = s.amax(dim=-1, keepdim=True) - s.amin(dim=-1, keepdim=True)
    return (s - m) / (r + NORM_EPS)


def mlp_weights(params, s, *, bf16: bool = False):
    """Softmax weights of stencils ``s[..., 5]``. With ``bf16`` the inputs and
    weights are rounded to bfloat16 (FP32 accumulation) and each hidden layer
    applies tanh to the bfloat16-rounded pre-activation with a bfloat16 result,
    as the tensor-core inference kernel does (tanh.approx.bf16x2)."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    x = _bf16(normalise(s), bf16)
    h1 = _bf16(torch.tanh(_bf16(x @ _bf16(W1, bf16).T + _bf16(b1, bf16), bf16)), bf16)
    h2 = _bf16(torch.tanh(_bf16(h1 @ _bf16(W2, bf16).T + b2, bf16)), bf16)
    z = h2 @ _bf16(W3, bf16).T + b3
    return torch.softmax(z, dim=-1)


def substencils(s: torch.Tensor) -> torch.Tensor:
    """The three WENO-JS5 sub-stencil values at the right face
    (``src/pyshocks/weno.py:231-239``)."""
    s0, s1, s2, s3, s4 = s.unbind(-1)
    return torch.stack([(2 * s0 - 7 * s1 + 11 * s2) / 6,
                        (-s1 + 5 * s2 + 2 * s3) / 6,
                        (2 * s2 + 5 * s3 - s4) / 6], dim=-1)


def js_weights(s: torch.Tensor, eps: float) -> torch.Tensor:
    """WENO-JS5 weights of the right face (``src/pyshocks/weno.py:247-256``)."""
    s0, s1, s2, s3, s4 = s.unbind(-1)
    b0 = 13 / 12 * (s0 - 2 * s1 + s2) ** 2 + 0.25 * (s0 - 4 * s1 + 3 * s2) ** 2
    b1 = 13 / 12 * (s1 - 2 * s2 + s3) ** 2 + 0.25 * (s1 - s3) ** 2
    b2 = 13 / 12 * (s2 - 2 * s3 + s4) ** 2 + 0.25 * (3 * s2 - 4 * s3 + s4) ** 2
    a = torch.stack([_D53[0] / (eps + b0) ** 2, _D53[1] / (eps + b1) ** 2,
                     _D53[2] / (eps + b2) ** 2], dim=-1)
    return a / a.sum(dim=-1, keepdim=True)


def face_value(params, s, *, eps: float, tau: float, band: float, dev: float = 0.5,
               bf16: bool = False, return_fallback: bool = False):
    """Learned face value of stencils ``s[..., 5]`` with the WENO-JS fallback."""
    w = mlp_weights(params, s, bf16=bf16)
    wjs = js_weights(s, eps)
    excess = torch.sum(w * (wjs < tau).to(w.dtype), dim=-1)
    fb = (excess > band) | (torch.amax(torch.abs(w - wjs), dim=-1) > dev)
    w = torch.where(fb[..., None], wjs, w)
    v = torch.sum(w * substencils(s), dim=-1)
    return (v, fb) if return_fallback else v


def stencils_periodic(u: torch.Tensor):
    """Right-face stencils (v_{i-2..i+2}) and mirrored left-face stencils
    (v_{i+2..i-2}) of every cell of periodic rows ``u[B, N]``."""
    idx = torch.arange(-2, 3)
    n = u.shape[-1]
    cols = (torch.arange(n)[:, None] + idx[None, :]) % n
    sr = u[..., cols]
    sl = torch.flip(sr, dims=(-1,))
    return sl, sr


def learned_recon(u: torch.Tensor, weights: dict, eps: float):
    """``(ul, ur)`` of every cell for the torch oracle's ``face_flux``."""
    sl, sr = stencils_periodic(u)
    kw = dict(eps=eps, tau=weights["tau"], band=weights["band"], dev=weights.get("dev", 0.5),
              bf16=weights.get("bf16", False))
    return face_value(weights["params"], sl, **kw), face_value(weights["params"], sr, **kw)


def training_loss(params, s, target, weight, reg: float = 0.0):
    """Weighted squared face-value error of the raw network (no fallback) plus
    the pull toward the ideal weights:
    ``sum_i [w_i (sum_k omega_k uhat_k - target_i)^2 + reg |omega_i - d|^2] / n``."""
    w = mlp_weights(params, s)
    v = torch.sum(w * substencils(s), dim=-1)
    d = torch.tensor(_D53, dtype=w.dtype)
    return (torch.sum(weight * (v - target) ** 2) + reg * torch.sum((w - d) ** 2)) / s.shape[0]


def init_params(seed: int = 0, dtype=torch.float32) -> torch.Tensor:
    """Glorot-uniform weights, zero biases, and a last-layer bias that puts the
    untrained network's softmax at the ideal weights (1, 6, 3)/10."""
    g = torch.Generator().manual_seed(seed)
    parts = []
    for fan_out, fan_in in ((N_H, N_IN), (N_H, N_H), (N_OUT, N_H)):
        lim = (6.0 / (fan_in + fan_out)) ** 0.5
        parts.append((torch.rand(fan_out, fan_in, generator=g, dtype=torch.float64) * 2 - 1) * lim)
        parts.append(torch.zeros(fan_out, dtype=torch.float64))
    p = torch.cat([x.reshape(-1) for x in parts])
    p[-3:] = torch.log(torch.tensor(_D53, dtype=torch.float64))
    return p.to(dtype)
