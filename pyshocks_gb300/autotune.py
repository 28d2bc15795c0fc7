"""Launch-shape autotuner for batched plans.

The batched step kernel has two free shape parameters: the tile length (cells
per work item; the halo of the three fused stages is fixed by the stencil
reach, 9 cells rounded up for 16-byte alignment) and the number of CTAs per SM
of the persistent grid. Short tiles waste work on halo recompute; long tiles
cut the number of work items below the resident CTAs and leave SMs idle on
small batches; more CTAs per SM hide latency until registers or shared memory
run out. :func:`tune` times every feasible candidate on the caller's batch
(CUDA events around a few graph-captured steps) and returns the fastest.
Results are cached per GPU, scheme, precision and batch shape, in memory and
in a JSON file (``$PYSHOCKS_GB300_CACHE`` or
``~/.cache/pyshocks_gb300/autotune.json``).
"""

from __future__ import annotations

import json
import os
import pathlib
from dataclasses import asdict, dataclass, field
from typing import Sequence

import numpy as np
import torch

#: candidate tile lengths (multiples of 16 cells keep every window 16-byte aligned)
TILES = (512, 1024, 2048, 4096)
#: candidate resident CTAs per SM (0: the plan's own choice from shared memory)
CTAS_PER_SM = (0, 1, 2, 3, 4)
#: the shared memory one SM offers to resident CTAs (bytes)
SMEM_PER_SM = 227 * 1024

_MEMO: dict[str, "TuneResult"] = {}


@dataclass
class TuneResult:
    tile: int
    ctas_per_sm: int
    ms_per_step: float  # forward step, or forward + reverse step for adjoint plans
    table: list = field(default_factory=list)  # (tile, ctas_per_sm, ms) of every candidate


def cache_path() -> pathlib.Path:
    env = os.environ.get("PYSHOCKS_GB300_CACHE")
    if env:
        return pathlib.Path(env)
    return pathlib.Path.home() / ".cache" / "pyshocks_gb300" / "autotune.json"


def shape_key(scheme, sizes: Sequence[int], dtype: torch.dtype, device) -> str:
    """Cache key: GPU name, scheme and reconstruction classes, dtype, and the
    batch shape (instance count and the histogram of log2 sizes)."""
    sizes = np.asarray(sizes, dtype=np.int64)
    logs = np.floor(np.log2(np.maximum(sizes, 1))).astype(int)
    hist = {int(k): int(v) for k, v in zip(*np.unique(logs, return_counts=True))}
    rec = getattr(scheme, "rec", None)
    name = torch.cuda.get_device_name(torch.device(device))
    return json.dumps([name, type(scheme).__name__, type(rec).__name__ if rec is not None else None,
                       str(dtype), int(sizes.size), hist], sort_keys=True)


#: static shared memory of the kernels with the learned reconstruction: the
#: staged network fragments (forward; forward and backward in the reverse step)
LEARNED_STATIC = 3584
LEARNED_STATIC_ADJOINT = 6400


def _smem_bytes(tile: int, dtype: torch.dtype, learned: bool = False, weno5: bool = False) -> int:
    # the step tile's shared memory: 7 double arrays of the window (halo 10),
    # or for the learned reconstruction the double window plus 6 float arrays
    # (the face-flux array at least 1028 floats); for float32 states (halo 12)
    # 6 float arrays with WENO-JS5, else 8
    if dtype == torch.float64:
        w = tile + 20
        if learned:
            return w * 8 + (5 * w + max(w, 1028)) * 4 + LEARNED_STATIC
        return w * 7 * 8
    return (6 if weno5 else 8) * (tile + 24) * 4 + (LEARNED_STATIC if learned else 0)


def _adjoint_smem_bytes(tile: int, dtype: torch.dtype, learned: bool = False) -> int:
    # the reverse step: 24 windows (halo 20) of the state type, or for float64
    # with the learned reconstruction 22 float windows
    w = tile + 40
    extra = LEARNED_STATIC_ADJOINT if learned else 0
    if dtype == torch.float64:
        return w * (22 * 4 if learned else 24 * 8) + extra
    return w * 24 * 4 + extra


def candidates(dtype: torch.dtype, max_cells: int, learned: bool = False,
               adjoint: bool = False, weno5: bool = False) -> list[tuple[int, int]]:
    """(tile, ctas_per_sm) pairs whose shared memory fits one SM; tiles longer
    than twice the largest instance are skipped (they only add idle lanes);
    with ``adjoint`` only tiles whose reverse step fits too."""
    out = []
    for tile in TILES:
        if tile > max(2 * max_cells, TILES[0]):
            continue
        if adjoint and _adjoint_smem_bytes(tile, dtype, learned) > SMEM_PER_SM:
            continue
        per = _smem_bytes(tile, dtype, learned, weno5)
        if per > SMEM_PER_SM:
            continue
        for c in CTAS_PER_SM:
            if c and c * per > SMEM_PER_SM:
                continue
            out.append((tile, c))
    return out


def _load_file() -> dict:
    p = cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def _store_file(key: str, res: TuneResult) -> None:
    p = cache_path()
    try:
        data = _load_file()
        data[key] = asdict(res)
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
        tmp.replace(p)
    except OSError:
        pass  # a read-only home is not an error: the in-memory result stands


def tune(scheme, sizes: Sequence[int], dx, *, dtype: torch.dtype = torch.float64,
         theta: float = 1.0, u0: torch.Tensor | None = None, steps: int = 4,
         device="cuda", use_cache: bool = True, adjoint: bool = False) -> TuneResult:
    """Time every candidate shape on this batch and return the fastest.

    :arg adjoint: keep to tiles the reverse step can run and time a short
        checkpointed forward solve plus its reverse sweep instead of forward
        steps (plans that record a dt history for the adjoint, whose reverse
        step dominates and prefers other shapes than the forward).

    :arg u0: packed state to step from (default: a smooth state of O(1)
        values); the step cost does not depend on the data except through the
        learned reconstruction's fallback branches.
    """
    from pyshocks_gb300.batched import BatchedSolver, pack_offsets

    key = shape_key(scheme, sizes, dtype, device) + (":adjoint" if adjoint else "")
    if use_cache:
        if key in _MEMO:
            return _MEMO[key]
        hit = _load_file().get(key)
        if hit is not None:
            res = TuneResult(**hit)
            _MEMO[key] = res
            return res
    sizes = np.asarray(sizes, dtype=np.int64)
    if u0 is None:
        off = pack_offsets(sizes)
        idx = torch.arange(int(off[-1]), device=device, dtype=torch.float64)
        u0 = 0.5 + 0.3 * torch.sin(0.01 * idx)
    stream = torch.cuda.Stream(device=device)
    table = []
    k = 2 * max(1, steps // 2)
    learned = type(getattr(scheme, "rec", None)).__name__ == "LearnedWENO"
    weno5 = type(getattr(scheme, "rec", None)).__name__ == "WENOJS53"
    for tile, cps in candidates(dtype, int(sizes.max()), learned, adjoint, weno5):
        if learned and tile < 512:
            continue  # the learned phase's warp scratch needs 512-cell tiles
        solver = BatchedSolver(scheme, sizes, dx, theta=theta, dtype=dtype, tile=tile,
                               ctas_per_sm=cps, device=device, max_steps=k if adjoint else 0)
        with torch.cuda.stream(stream):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            if adjoint:
                from pyshocks_gb300.adjoint import CheckpointedSolve

                cs = CheckpointedSolve(solver, k)
                cs.backward(cs.forward(u0))  # warm-up
                e0.record(stream)
                cs.backward(cs.forward(u0))
                e1.record(stream)
                e1.synchronize()
                del cs
            else:
                solver.reset(u0)
                solver.step(2, graph=True)
                e0.record(stream)
                solver.step(k, graph=True)
                e1.record(stream)
                e1.synchronize()
        if solver.status() == 0:
            table.append((tile, cps, e0.elapsed_time(e1) / k))
        del solver
    if not table:
        raise RuntimeError("no launch shape ran cleanly")
    best = min(table, key=lambda r: r[2])
    res = TuneResult(tile=best[0], ctas_per_sm=best[1], ms_per_step=best[2], table=table)
    _MEMO[key] = res
    if use_cache:
        _store_file(key, res)
    return res
