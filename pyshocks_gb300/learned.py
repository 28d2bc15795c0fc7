"""Learned WENO weights: reconstruction, training data and training loop.

The network (``csrc/learned.cuh``) maps the normalised 5-point stencil of a
face to the three WENO-JS5 sub-stencil weights through a softmax, so the face
value stays a convex combination of the sub-stencil values and the flux stays
conservative. It plugs into the reference's reconstruction slot
(``src/pyshocks/reconstruction.py:79-119``) as :class:`LearnedWENO`. Plain
WENO-JS is the per-face fallback wherever the network leaves the trust band:
more than ``band`` of its weight on sub-stencils whose JS weight is below
``tau`` (sub-stencils across a discontinuity), or any weight more than ``dev``
away from the JS weight. ``dev`` = 0.8 keeps the long-run overshoots at the
level of the network-free linear weights (a cap of 0.5 suppressed them but
raised the L1 error of the trained network by 32 %; no cap doubled them).

Training pairs come from the plain solver itself: fine-grid runs (N = 4096)
restricted to the coarse grid (N = 256, 16-cell averages) give coarse stencils,
and the fine solution gives the face value each stencil should reconstruct.
Training runs on the GPU with the hand-written loss/gradient and Adam kernels.
"""

from __future__ import annotations

import math
import pathlib
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np
import torch

from pyshocks_gb300 import _lib as L
from pyshocks_gb300.reconstruction import Reconstruction

N_PARAMS = 1347
_D53 = (0.1, 0.6, 0.3)


def init_params(seed: int = 0, device="cuda") -> torch.Tensor:
    """Glorot-uniform weights, zero hidden biases and an output bias of
    ``log(d)``, so an untrained network starts near the ideal weights
    ``d = (0.1, 0.6, 0.3)`` of WENO-JS5 (``src/pyshocks/weno.py:242``)."""
    g = torch.Generator().manual_seed(seed)
    parts = []
    for fan_out, fan_in in ((32, 5), (32, 32), (3, 32)):
        lim = math.sqrt(6.0 / (fan_in + fan_out))
        parts.append((torch.rand(fan_out, fan_in, generator=g, dtype=torch.float64) * 2 - 1) * lim)
        parts.append(torch.zeros(fan_out, dtype=torch.float64))
    p = torch.cat([x.reshape(-1) for x in parts])
    p[-3:] = torch.log(torch.tensor(_D53, dtype=torch.float64))
    assert p.numel() == N_PARAMS
    return p.to(device=device, dtype=torch.float32)


#: floor of the stencil range in the network's input normalisation: features
#: far below it (rounding noise on flat states) reach the network as ~0 inputs,
#: as WENO-JS's eps makes such features linear
NORM_EPS = 1.0e-5

DEFAULT_PARAMS = pathlib.Path(__file__).resolve().parent / "data" / "mlp_weno_burgers_advection.npy"


def load_default_params(device="cuda") -> torch.Tensor:
    """The network trained by :func:`train_default` (committed with the package;
    regenerate with ``python -m pyshocks_gb300.learned``). Falls back to the
    untrained initialisation when the file is absent."""
    if DEFAULT_PARAMS.exists():
        return torch.tensor(np.load(DEFAULT_PARAMS), dtype=torch.float32, device=device)
    return init_params(device=device)


@dataclass(frozen=True, eq=False)
class LearnedWENO(Reconstruction):
    """Learned-weight WENO reconstruction. With float64 states the stencil
    differences and the network run in float32/bfloat16 and the face value is
    assembled in float64 (``v_c + correction``)."""

    params: torch.Tensor = field(default_factory=lambda: init_params())
    eps: float = 1.0e-6
    tau: float = 1.0e-2
    band: float = 0.1
    dev: float = 0.8
    #: floor of the stencil range in the input normalisation
    #: ``(s - mean) / (range + norm_eps)`` (the network's counterpart of eps)
    norm_eps: float = NORM_EPS

    code = L.SHK_REC_LEARNED

    @property
    def order(self) -> int:
        return 3

    @property
    def stencil_width(self) -> int:
        return 3

    def __post_init__(self):
        p = self.params
        if not (isinstance(p, torch.Tensor) and p.is_cuda and p.dtype == torch.float32
                and p.numel() == N_PARAMS and p.is_contiguous()):
            raise ValueError(f"params must be a contiguous float32 CUDA tensor of {N_PARAMS}")


def c_scheme_fields(rec: LearnedWENO, s: L.ShkScheme) -> None:
    s.mlp = rec.params.data_ptr()
    s.tau = float(rec.tau)
    s.band = float(rec.band)
    s.dev = float(rec.dev)
    s.norm_eps = float(rec.norm_eps)


def face_values(scheme, stencils: torch.Tensor) -> torch.Tensor:
    """Learned ``(right, left)`` face values ``[n, 2]`` of cell stencils
    ``v_{c-2..c+2}`` (``stencils[n, 5]``, float32, CUDA) with the tensor-core
    path and trust band of the flux kernel."""
    st = stencils.contiguous()
    out = torch.empty((st.shape[0], 2), dtype=torch.float32, device=st.device)
    L.check(L.lib().shk_learned_faces_f32(scheme.c_scheme(1.0), st.data_ptr(), out.data_ptr(),
                                          st.shape[0], L.stream_handle()), "learned_faces")
    return out


# {{{ training data


def _stencils_periodic(U: torch.Tensor) -> torch.Tensor:
    """Cell stencils ``U_{c-2..c+2}`` of every cell of periodic rows ``U[B, N]``."""
    n = U.shape[-1]
    idx = (torch.arange(n, device=U.device)[:, None] + torch.arange(-2, 3, device=U.device)) % n
    return U[:, idx]


def _fine_face_values(F: torch.Tensor, r: int):
    """Values at the coarse faces from fine cell averages ``F[B, N r]``: the
    fourth-order interpolant (-F_{j-2} + 7 F_{j-1} + 7 F_j - F_{j+1}) / 12 at the
    fine face between cells j-1 and j. Returns (left faces, right faces) of each
    coarse cell."""
    nf = F.shape[-1]
    j = torch.arange(0, nf, r, device=F.device)  # left face of coarse cell c is fine face r c

    def at(k):
        return F[:, (j[None, :] + k) % nf]

    left = (-at(-2) + 7 * at(-1) + 7 * at(0) - at(1)) / 12
    right = torch.roll(left, shifts=-1, dims=-1)
    return left, right


def generate_pairs(
    *,
    n_coarse: int = 256,
    ratio: int = 16,
    n_ics: int = 256,
    snapshots: int = 16,
    steps_between: int = 256,
    seed: int = 0,
    equations: Sequence[str] = ("burgers", "advection"),
    device="cuda",
):
    """Training pairs from the plain FP64 solver: fine runs at ``n_coarse *
    ratio`` cells (Rusanov + WENO-JS5, eps 1e-6) from 0.5 + sin(pi x)-like and
    random-Fourier initial conditions, sampled every ``steps_between`` steps and
    restricted to ``n_coarse`` cells. Returns float32 cell samples
    ``(stencils[n, 5], targets[n, 2], weights[n])``: the stencil
    ``U_{c-2..c+2}``, the fine-grid values at the cell's right and left faces,
    and the weight ``1 / (range + 1e-3)^2`` that makes the loss a
    range-normalised face error."""
    from pyshocks_gb300 import burgers, reconstruction
    from pyshocks_gb300.batched import BatchedSolver

    nf = n_coarse * ratio
    rng = np.random.default_rng(seed)
    rec = reconstruction.make_reconstruction_from_name("wenojs53", eps=1.0e-6)
    out_s, out_t, out_w = [], [], []
    for eq in equations:
        scheme = burgers.Rusanov(rec=rec) if eq == "burgers" else burgers.AdvectionRusanov(rec=rec)
        u0 = _initial_conditions(rng, n_ics, nf, device)
        solver = BatchedSolver(scheme, [nf] * n_ics, 2.0 / nf, theta=1.0)
        solver.reset(u0.reshape(-1))
        for _ in range(snapshots):
            solver.step(steps_between)
            F = solver.u.reshape(n_ics, nf)
            U = F.reshape(n_ics, n_coarse, ratio).mean(dim=-1)
            sc = _stencils_periodic(U).reshape(-1, 5)
            tl, tr = _fine_face_values(F, ratio)
            rngs = sc.amax(dim=-1) - sc.amin(dim=-1)
            out_s.append(sc.float())
            out_t.append(torch.stack([tr.reshape(-1), tl.reshape(-1)], dim=-1).float())
            out_w.append((1.0 / (rngs + 1.0e-3) ** 2).float())
        solver.check_status()
        del solver
    return torch.cat(out_s), torch.cat(out_t), torch.cat(out_w)


def _initial_conditions(rng, B: int, n: int, device) -> torch.Tensor:
    """Exact cell averages of a mix of ``m + A sin(k pi x + phi)`` (the family of
    0.5 + sin(pi x)) and random 8-mode Fourier series with 0-3 jumps."""
    f = torch.linspace(-1.0, 1.0, n + 1, dtype=torch.float64, device=device)
    fl, fr = f[:-1], f[1:]
    h = 2.0 / n
    rows = []
    for b in range(B):
        if b % 2 == 0:
            m = rng.uniform(-0.5, 0.5) if b else 0.5
            A = rng.uniform(0.3, 1.2) if b else 1.0
            k = int(rng.integers(1, 4)) if b else 1
            ph = rng.uniform(0, 2 * np.pi) if b else 0.0
            u = m + A * (torch.cos(k * np.pi * fl + ph) - torch.cos(k * np.pi * fr + ph)) / (k * np.pi * h)
        else:
            m = rng.uniform(-0.5, 0.5)
            u = torch.full_like(fl, m)
            for k in range(1, 9):
                a = rng.normal() / k**2
                ph = rng.uniform(0, 2 * np.pi)
                u += a * (torch.cos(k * np.pi * fl + ph) - torch.cos(k * np.pi * fr + ph)) / (k * np.pi * h)
            for _ in range(int(rng.integers(0, 4))):
                hj, xj = rng.uniform(-1, 1), rng.uniform(-1, 1)
                u += hj * torch.clamp((fr - xj) / h, 0.0, 1.0)
        rows.append(u)
    return torch.stack(rows)


# }}}


# {{{ training


class Trainer:
    """Adam on the MLP parameters with the CUDA loss/gradient kernel."""

    def __init__(self, params: torch.Tensor, *, lr: float = 2.0e-3, betas=(0.9, 0.999),
                 eps: float = 1.0e-8, max_batch: int = 1 << 16, reg: float = 1.0e-3,
                 norm_eps: float | None = None):
        self.lib = L.lib()
        self.params = params
        self.m = torch.zeros_like(params)
        self.v = torch.zeros_like(params)
        self.grad = torch.zeros_like(params)
        self.loss_dev = torch.zeros((), dtype=torch.float64, device=params.device)
        self.lr, self.betas, self.eps = lr, betas, eps
        self.step_count = 0
        self.ws = torch.empty(int(self.lib.shk_mlp_workspace_bytes(max_batch)), dtype=torch.uint8,
                              device=params.device)
        self.max_batch = max_batch
        self.reg = float(reg)
        self.norm_eps = float(NORM_EPS if norm_eps is None else norm_eps)

    def loss_and_grad(self, s: torch.Tensor, t: torch.Tensor, w: torch.Tensor) -> torch.Tensor:
        n = s.shape[0]
        need = int(self.lib.shk_mlp_workspace_bytes(n))
        if need > self.ws.numel():
            self.ws = torch.empty(need, dtype=torch.uint8, device=self.params.device)
        L.check(self.lib.shk_mlp_loss_grad_f32(
            self.params.data_ptr(), s.data_ptr(), t.data_ptr(), w.data_ptr(), n, self.reg,
            self.norm_eps, self.grad.data_ptr(), self.loss_dev.data_ptr(), self.ws.data_ptr(), self.ws.numel(),
            L.stream_handle()), "mlp_loss_grad")
        return self.loss_dev

    def step(self, s, t, w, lr: float | None = None) -> torch.Tensor:
        loss = self.loss_and_grad(s, t, w)
        self.step_count += 1
        L.check(self.lib.shk_mlp_adam_f32(
            self.params.data_ptr(), self.grad.data_ptr(), self.m.data_ptr(), self.v.data_ptr(),
            float(lr if lr is not None else self.lr), float(self.betas[0]), float(self.betas[1]),
            float(self.eps), self.step_count, L.stream_handle()), "mlp_adam")
        return loss

    def fit(self, s, t, w, *, epochs: int = 1, batch: int = 1 << 15, seed: int = 0,
            lr_final: float | None = None) -> list[float]:
        """Minibatch Adam over the pairs; returns the mean loss of each epoch."""
        n = s.shape[0]
        g = torch.Generator(device=s.device).manual_seed(seed)
        hist = []
        total = epochs * max(1, n // batch)
        it = 0
        for _ in range(epochs):
            perm = torch.randperm(n, device=s.device, generator=g)
            acc = torch.zeros((), dtype=torch.float64, device=s.device)
            nb = 0
            for i in range(0, n - batch + 1, batch):
                idx = perm[i:i + batch]
                lr = self.lr
                if lr_final is not None:  # cosine decay
                    lr = lr_final + 0.5 * (self.lr - lr_final) * (1 + math.cos(math.pi * it / total))
                acc += self.step(s[idx].contiguous(), t[idx].contiguous(), w[idx].contiguous(), lr)
                nb += 1
                it += 1
            hist.append(float(acc) / max(nb, 1))
        return hist


# }}}


def train_default(*, n_ics: int = 640, epochs: int = 64, reg: float = 0.02, seed: int = 0,
                  lr: float = 1.0e-2, batch: int = 32768):
    """Train the default network: 5.2e6 cells (1.05e7 face targets; N = 256
    restricted from N = 4096, Burgers and linear advection, 0.5 + sin(pi x)-like and
    random-Fourier initial conditions), Adam with cosine decay to 1e-4.
    Returns ``(params, loss history)``. The committed default was made with
    these arguments and ``NORM_EPS`` (the loss, face error plus the pull
    toward the ideal weights, falls from 5.8e-4 to 3.6e-4)."""
    s, t, w = generate_pairs(n_coarse=256, ratio=16, n_ics=n_ics, snapshots=16,
                             steps_between=256, seed=seed)
    params = init_params(seed=seed)
    tr = Trainer(params, lr=lr, reg=reg, norm_eps=NORM_EPS)
    hist = tr.fit(s, t, w, epochs=epochs, batch=batch, lr_final=1.0e-4, seed=seed)
    return params, hist


if __name__ == "__main__":
    p, h = train_default()
    DEFAULT_PARAMS.parent.mkdir(exist_ok=True)
    np.save(DEFAULT_PARAMS, p.cpu().numpy())
    print("losses", h)

