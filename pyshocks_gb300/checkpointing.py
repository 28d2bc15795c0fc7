"""Checkpoints for the adjoint (mirrors ``src/pyshocks/checkpointing.py``).

``InMemoryCheckpoint`` keeps device tensors (no host copies). The adjoint of
the batched path uses its own device-resident sqrt(n) checkpoint pool.
"""

from __future__ import annotations

import pathlib
from abc import ABC
from dataclasses import dataclass, field
from functools import singledispatch
from typing import Any

import numpy as np
import torch


@dataclass
class Checkpoint(ABC):
    """``src/pyshocks/checkpointing.py:36-72``."""

    basename: str


@singledispatch
def save(chk: Checkpoint, idx: int, values: dict[str, Any]) -> None:
    """``src/pyshocks/checkpointing.py:75-81``."""
    raise NotImplementedError(type(chk).__name__)


@singledispatch
def load(chk: Checkpoint, idx: int) -> dict[str, Any]:
    """``src/pyshocks/checkpointing.py:84-95``."""
    raise NotImplementedError(type(chk).__name__)


@dataclass
class InMemoryCheckpoint(Checkpoint):
    """``src/pyshocks/checkpointing.py:101-140``."""

    storage: dict[tuple[str, int], dict[str, Any]] = field(default_factory=dict, repr=False)


@save.register(InMemoryCheckpoint)
def _save_in_memory(chk: InMemoryCheckpoint, idx: int, values: dict[str, Any]) -> None:
    key = (chk.basename, idx)
    if key in chk.storage:
        raise KeyError(f"Cannot save checkpoint '{key}'. Key already exists.")
    chk.storage[key] = values


@load.register(InMemoryCheckpoint)
def _load_in_memory(chk: InMemoryCheckpoint, idx: int) -> dict[str, Any]:
    key = (chk.basename, idx)
    if key not in chk.storage:
        raise KeyError(f"Cannot load checkpoint '{key}'. Key does not exist.")
    return chk.storage[key]


@dataclass
class NumpyCheckpoint(Checkpoint):
    """``.npz`` files with keys ``m``, ``t``, ``u`` (``src/pyshocks/checkpointing.py:209-254``).

    The reference raises when the target file does *not* exist
    (``checkpointing.py:233-234``), so a fresh save always fails there; here a
    save refuses to overwrite an existing file and a load requires one.
    """

    dirname: pathlib.Path = field(default_factory=pathlib.Path.cwd)

    def path(self, idx: int) -> pathlib.Path:
        return pathlib.Path(self.dirname) / f"{self.basename}_{idx:09d}.npz"


@save.register(NumpyCheckpoint)
def _save_npz(chk: NumpyCheckpoint, idx: int, values: dict[str, Any]) -> None:
    p = chk.path(idx)
    if p.exists():
        raise FileExistsError(f"Cannot save checkpoint '{p}'. File already exists.")
    arrays = {k: (v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v))
              for k, v in values.items()}
    np.savez(p, **arrays)


@load.register(NumpyCheckpoint)
def _load_npz(chk: NumpyCheckpoint, idx: int) -> dict[str, Any]:
    p = chk.path(idx)
    if not p.exists():
        raise FileNotFoundError(f"Cannot load checkpoint '{p}'. File does not exist.")
    with np.load(p) as data:
        return {k: data[k] for k in data.files}
