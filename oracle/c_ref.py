"""ctypes wrapper of ``oracle/shocks_ref.c`` (the C restatement of the oracle).

Test infrastructure and CPU baseline only; see ``oracle/shocks_ref.c``.
"""

from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "libshocks_ref.so"


def build(force: bool = False) -> pathlib.Path:
    src = HERE / "shocks_ref.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "-B" if force else "libshocks_ref.so"],
                       check=True)
    return LIB


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(str(LIB))
        _lib.ref_run_batch.restype = ctypes.c_int
        _lib.ref_run_batch.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                       ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32]
    return _lib


def run_batch(u0: np.ndarray, offsets: np.ndarray, dx: np.ndarray, *, theta: float = 1.0,
              eps: float = 1.0e-6, nsteps: int = 1, nthreads: int = 0,
              want_dts: bool = False):
    """Fixed-count Burgers WENO-JS5/Rusanov/SSPRK33 run of a packed batch.
    Returns ``(u, dts, threads_used)``."""
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    dxa = np.ascontiguousarray(dx, dtype=np.float64)
    B = off.size - 1
    dts = np.zeros((nsteps, B)) if want_dts else None
    used = lib().ref_run_batch(u.ctypes.data, off.ctypes.data, B, dxa.ctypes.data, theta, eps,
                               nsteps, dts.ctypes.data if dts is not None else None,
                               int(nthreads or os.cpu_count() or 1))
    return u, dts, used
