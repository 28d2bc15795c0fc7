"""Checkpoints for the adjoint (mirrors ``src/pyshocks/checkpointing.py``).

``InMemoryCheckpoint`` keeps device tensors (no host copies). The adjoint of
the batched path uses its own device-resident sqrt(n) checkpoint pool.

The interface is the reference's: ``save(chk, idx, values)``,
``load(chk, idx, include=None)``, ``idx in chk`` and ``chk.index_to_key(idx)``,
with ``KeyError`` for a duplicate save or a missing load.
"""

from __future__ import annotations

import pathlib
from abc import ABC, abstractmethod
from collections.abc import Hashable
from dataclasses import dataclass, field
from functools import singledispatch
from typing import Any

import numpy as np
import torch


class CheckpointExistsError(FileExistsError, KeyError):
    """Saving over an existing ``.npz`` checkpoint: a ``KeyError`` as in the
    reference, and a ``FileExistsError``."""


class CheckpointNotFoundError(FileNotFoundError, KeyError):
    """Loading a missing ``.npz`` checkpoint: a ``KeyError`` as in the
    reference, and a ``FileNotFoundError``."""


@dataclass(frozen=True)
class Checkpoint(ABC):
    """``src/pyshocks/checkpointing.py:36-72``."""

    basename: str

    @abstractmethod
    def index_to_key(self, i: int) -> Hashable:
        """The key of checkpoint *i* in the storage backend."""

    @abstractmethod
    def __contains__(self, i: int) -> bool:
        pass


@singledispatch
def save(chk: Checkpoint, idx: int, values: dict[str, Any]) -> None:
    """``src/pyshocks/checkpointing.py:75-81``."""
    raise NotImplementedError(type(chk).__name__)


@singledispatch
def load(chk: Checkpoint, idx: int, *, include: tuple[str, ...] | None = None) -> dict[str, Any]:
    """``src/pyshocks/checkpointing.py:84-95``: the values saved at *idx*, only
    the keys in *include* if given."""
    raise NotImplementedError(type(chk).__name__)


def _select(values: dict[str, Any], include: tuple[str, ...] | None) -> dict[str, Any]:
    return values if include is None else {k: v for k, v in values.items() if k in include}


@dataclass(frozen=True)
class InMemoryCheckpoint(Checkpoint):
    """``src/pyshocks/checkpointing.py:101-140``."""

    storage: dict[Hashable, dict[str, Any]] = field(default_factory=dict, repr=False)

    def index_to_key(self, i: int) -> Hashable:
        return (self.basename, i)

    def __contains__(self, i: int) -> bool:
        return self.index_to_key(i) in self.storage


@save.register(InMemoryCheckpoint)
def _save_in_memory(chk: InMemoryCheckpoint, idx: int, values: dict[str, Any]) -> None:
    key = chk.index_to_key(idx)
    if key in chk.storage:
        raise KeyError(f"Cannot set existing checkpoint at {idx!r}.")
    chk.storage[key] = values


@load.register(InMemoryCheckpoint)
def _load_in_memory(chk: InMemoryCheckpoint, idx: int, *,
                    include: tuple[str, ...] | None = None) -> dict[str, Any]:
    key = chk.index_to_key(idx)
    if key not in chk.storage:
        raise KeyError(f"Cannot find checkpoint at index {idx!r}.")
    return _select(chk.storage[key], include)


@dataclass(frozen=True)
class NumpyCheckpoint(Checkpoint):
    """``.npz`` files ``<dirname>/<basename>_<idx:09d>.npz`` with the saved keys
    (``m``, ``t``, ``u`` from the steppers), ``src/pyshocks/checkpointing.py:209-254``.

    The reference raises when the target file does *not* exist
    (``checkpointing.py:233-234``), so a fresh save always fails there; here a
    save refuses to overwrite an existing file and a load requires one. Device
    tensors are copied to the host on save; loads return NumPy arrays.
    """

    dirname: pathlib.Path = field(default_factory=pathlib.Path.cwd)

    def index_to_key(self, i: int) -> pathlib.Path:
        return pathlib.Path(self.dirname) / f"{self.basename}_{i:09d}.npz"

    def __contains__(self, i: int) -> bool:
        return self.index_to_key(i).exists()

    def path(self, idx: int) -> pathlib.Path:
        return self.index_to_key(idx)


@save.register(NumpyCheckpoint)
def _save_npz(chk: NumpyCheckpoint, idx: int, values: dict[str, Any]) -> None:
    p = chk.index_to_key(idx)
    if p.exists():
        raise CheckpointExistsError(f"Cannot set existing checkpoint at {idx!r} ({p}).")
    arrays = {k: (v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v))
              for k, v in values.items()}
    np.savez(p, **arrays)


@load.register(NumpyCheckpoint)
def _load_npz(chk: NumpyCheckpoint, idx: int, *,
              include: tuple[str, ...] | None = None) -> dict[str, Any]:
    p = chk.index_to_key(idx)
    if not p.exists():
        raise CheckpointNotFoundError(f"Cannot find checkpoint at index {idx!r} ({p}).")
    with np.load(p, allow_pickle=False) as data:
        return _select({k: data[k] for k in data.files}, include)
