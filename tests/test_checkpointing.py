"""Checkpoint objects (``src/pyshocks/checkpointing.py``) on the host: the
reference's interface (``save``/``load``/``include``/``in``/``index_to_key``)
and errors (``KeyError`` for a duplicate save or a missing load), and the
``.npz`` files with the keys ``m``, ``t``, ``u`` (whose save, unlike the
reference's inverted existence check at ``checkpointing.py:233-234``,
writes a fresh file and refuses an existing one)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from pyshocks_gb300.checkpointing import (
    CheckpointExistsError,
    CheckpointNotFoundError,
    InMemoryCheckpoint,
    NumpyCheckpoint,
    load,
    save,
)


def test_in_memory_round_trip_and_errors():
    chk = InMemoryCheckpoint(basename="Iteration")
    for i in range(5):
        save(chk, i, {"m": i, "t": 0.1 * i, "u": torch.full((4,), float(i))})
    assert 3 in chk and 5 not in chk
    assert chk.index_to_key(3) == ("Iteration", 3)
    d = load(chk, 3)
    assert d["m"] == 3 and d["t"] == pytest.approx(0.3) and torch.all(d["u"] == 3.0)
    assert set(load(chk, 2, include=("u",))) == {"u"}
    with pytest.raises(KeyError):
        save(chk, 3, {"m": 3})
    with pytest.raises(KeyError):
        load(chk, 7)


def test_npz_round_trip_keys_and_file_names(tmp_path):
    chk = NumpyCheckpoint(basename="Iteration", dirname=tmp_path)
    u = torch.linspace(-1.0, 1.0, 17, dtype=torch.float64)
    save(chk, 0, {"m": 0, "t": 0.0, "u": u})
    save(chk, 12, {"m": 12, "t": 0.125, "u": 2.0 * u})
    assert chk.index_to_key(12) == tmp_path / "Iteration_000000012.npz"
    assert chk.index_to_key(12).exists() and 12 in chk and 1 not in chk
    with np.load(tmp_path / "Iteration_000000012.npz") as f:
        assert sorted(f.files) == ["m", "t", "u"]
    d = load(chk, 12)
    assert int(d["m"]) == 12 and float(d["t"]) == 0.125
    np.testing.assert_array_equal(d["u"], 2.0 * u.numpy())
    assert set(load(chk, 0, include=("t", "u"))) == {"t", "u"}


def test_npz_refuses_overwrite_and_missing_files(tmp_path):
    chk = NumpyCheckpoint(basename="Iteration", dirname=tmp_path)
    save(chk, 1, {"m": 1, "t": 0.5, "u": np.zeros(3)})
    with pytest.raises(FileExistsError):
        save(chk, 1, {"m": 1, "t": 0.5, "u": np.ones(3)})
    with pytest.raises(KeyError):  # the reference's exception type
        save(chk, 1, {"m": 1})
    np.testing.assert_array_equal(load(chk, 1)["u"], np.zeros(3))  # not overwritten
    with pytest.raises(FileNotFoundError):
        load(chk, 2)
    with pytest.raises(KeyError):
        load(chk, 2)
    assert issubclass(CheckpointExistsError, KeyError)
    assert issubclass(CheckpointNotFoundError, KeyError)
