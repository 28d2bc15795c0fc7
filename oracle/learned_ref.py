"""torch-CPU restatement of the learned-weight WENO reconstruction.

THIS IS TEST INFRASTRUCTURE (the oracle) for ``pyshocks_gb300/csrc/learned.cu``
and ``learned.cuh``: only tests use it, as the checker.

The method (no reference counterpart; it plugs into the reference's
reconstruction slot, ``src/pyshocks/reconstruction.py:79-119``): an MLP
5 -> 32 -> 32 -> 3 (tanh, tanh, softmax) maps the normalised 5-point stencil
``s = v_{c-2..c+2}`` of a cell to the weights of the WENO-JS5 sub-stencils
(``src/pyshocks/weno.py:206-244``) at its right face, ``omega_R = softmax(z)``;
the left face reuses the scores with its own ideal weights (as WENO-JS5 reuses
its smoothness indicators): ``omega_L = softmax(z2 - ln 3, z1, z0 + ln 3)``.
Each face value is the convex combination ``sum_k omega_k uhat_k`` of its
sub-stencil values, so the flux stays conservative. Where the network puts
more than ``band`` of a face's weight on sub-stencils that WENO-JS marks as
crossing a discontinuity (JS weight below ``tau``), or moves any weight more
than ``dev`` from the JS weight, that face uses the plain WENO-JS weights.

Parameter vector (1347 float32): W1[32,5], b1[32], W2[32,32], b2[32],
W3[3,32], b3[3], row-major.
"""

from __future__ import annotations

import torch

N_IN, N_H, N_OUT = 5, 32, 3
N_PARAMS = N_H * N_IN + N_H + N_H * N_H + N_H + N_OUT * N_H + N_OUT
NORM_EPS = 1.0e-5
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


def normalise(s: torch.Tensor, norm_eps: float = NORM_EPS) -> torch.Tensor:
    """``(s - mean) / (max - min + norm_eps)`` of stencils ``s[..., 5]``."""
    m = s.mean(dim=-1, keepdim=True)
    r = s.amax(dim=-1, keepdim=True) - s.amin(dim=-1, keepdim=True)
    return (s - m) / (r + norm_eps)


def logits(params, s, *, bf16: bool = False, norm_eps: float = NORM_EPS):
    """Network output ``z`` of cell stencils ``s[..., 5]``. With ``bf16`` the
    inputs and weights are rounded to bfloat16 (FP32 accumulation) and each
    hidden layer applies tanh to the bfloat16-rounded pre-activation with a
    bfloat16 result, as the tensor-core inference kernel does
    (tanh.approx.bf16x2)."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    x = _bf16(normalise(s, norm_eps), bf16)
    h1 = _bf16(torch.tanh(_bf16(x @ _bf16(W1, bf16).T + _bf16(b1, bf16), bf16)), bf16)
    h2 = _bf16(torch.tanh(_bf16(h1 @ _bf16(W2, bf16).T + b2, bf16)), bf16)
    return h2 @ _bf16(W3, bf16).T + b3


def mlp_weights(params, s, *, bf16: bool = False, norm_eps: float = NORM_EPS):
    """Right- and left-face softmax weights ``(omega_R, omega_L)`` of cell
    stencils ``s[..., 5]`` from one network evaluation."""
    z = logits(params, s, bf16=bf16, norm_eps=norm_eps)
    ln3 = torch.log(torch.tensor(3.0, dtype=z.dtype))
    zl = torch.stack([z[..., 2] - ln3, z[..., 1], z[..., 0] + ln3], dim=-1)
    return torch.softmax(z, dim=-1), torch.softmax(zl, dim=-1)


def substencils(s: torch.Tensor):
    """WENO-JS5 sub-stencil values at the right face (``src/pyshocks/weno.py:231-239``)
    and at the left face (the same formulas on the mirrored stencil)."""
    def right(q):
        q0, q1, q2, q3, q4 = q.unbind(-1)
        return torch.stack([(2 * q0 - 7 * q1 + 11 * q2) / 6,
                            (-q1 + 5 * q2 + 2 * q3) / 6,
                            (2 * q2 + 5 * q3 - q4) / 6], dim=-1)
    return right(s), right(torch.flip(s, dims=(-1,)))


def js_weights(s: torch.Tensor, eps: float):
    """WENO-JS5 weights of the right face (``src/pyshocks/weno.py:247-256``) and
    of the left face (the mirrored stencil: ideal weight d_k on beta_{2-k})."""
    s0, s1, s2, s3, s4 = s.unbind(-1)
    b0 = 13 / 12 * (s0 - 2 * s1 + s2) ** 2 + 0.25 * (s0 - 4 * s1 + 3 * s2) ** 2
    b1 = 13 / 12 * (s1 - 2 * s2 + s3) ** 2 + 0.25 * (s1 - s3) ** 2
    b2 = 13 / 12 * (s2 - 2 * s3 + s4) ** 2 + 0.25 * (3 * s2 - 4 * s3 + s4) ** 2
    r0, r1, r2 = 1 / (eps + b0) ** 2, 1 / (eps + b1) ** 2, 1 / (eps + b2) ** 2
    ar = torch.stack([_D53[0] * r0, _D53[1] * r1, _D53[2] * r2], dim=-1)
    al = torch.stack([_D53[0] * r2, _D53[1] * r1, _D53[2] * r0], dim=-1)
    return ar / ar.sum(dim=-1, keepdim=True), al / al.sum(dim=-1, keepdim=True)


def _band(w, wjs, tau, band, dev):
    excess = torch.sum(w * (wjs < tau).to(w.dtype), dim=-1)
    return (excess > band) | (torch.amax(torch.abs(w - wjs), dim=-1) > dev)


def cell_face_values(params, s, *, eps: float, tau: float, band: float, dev: float = 0.8,
                     bf16: bool = False, return_fallback: bool = False,
                     norm_eps: float = NORM_EPS):
    """Learned ``(right, left)`` face values of cell stencils ``s[..., 5]``
    with the per-face WENO-JS fallback."""
    wr, wl = mlp_weights(params, s, bf16=bf16, norm_eps=norm_eps)
    jr, jl = js_weights(s, eps)
    fr, fl = _band(wr, jr, tau, band, dev), _band(wl, jl, tau, band, dev)
    wr = torch.where(fr[..., None], jr, wr)
    wl = torch.where(fl[..., None], jl, wl)
    hr, hl = substencils(s)
    vr, vl = torch.sum(wr * hr, dim=-1), torch.sum(wl * hl, dim=-1)
    return ((vr, vl), (fr, fl)) if return_fallback else (vr, vl)


def stencils_periodic(u: torch.Tensor):
    """Cell stencils ``v_{i-2..i+2}`` of every cell of periodic rows ``u[B, N]``."""
    idx = torch.arange(-2, 3)
    n = u.shape[-1]
    cols = (torch.arange(n)[:, None] + idx[None, :]) % n
    return u[..., cols]


def learned_recon(u: torch.Tensor, weights: dict, eps: float):
    """``(ul, ur)`` of every cell for the torch oracle's ``face_flux``."""
    kw = dict(eps=eps, tau=weights["tau"], band=weights["band"], dev=weights.get("dev", 0.8),
              bf16=weights.get("bf16", False), norm_eps=weights.get("norm_eps", NORM_EPS))
    vr, vl = cell_face_values(weights["params"], stencils_periodic(u), **kw)
    return vl, vr


def training_loss(params, s, target, weight, reg: float = 0.0, norm_eps: float = NORM_EPS):
    """Weighted squared face-value error of the raw network (no fallback) over
    both faces of each cell, plus the pull toward the ideal weights:
    ``sum_i sum_F [w_i (sum_k omega_F,k uhat_F,k - T_F,i)^2 + reg |omega_F,i - d|^2] / (2 n)``
    with ``target[:, 0]`` / ``target[:, 1]`` the right / left face targets."""
    wr, wl = mlp_weights(params, s, norm_eps=norm_eps)
    hr, hl = substencils(s)
    vr, vl = torch.sum(wr * hr, dim=-1), torch.sum(wl * hl, dim=-1)
    d = torch.tensor(_D53, dtype=wr.dtype)
    err = weight * ((vr - target[:, 0]) ** 2 + (vl - target[:, 1]) ** 2)
    pull = torch.sum((wr - d) ** 2, dim=-1) + torch.sum((wl - d) ** 2, dim=-1)
    return (torch.sum(err) + reg * torch.sum(pull)) / (2 * s.shape[0])


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
