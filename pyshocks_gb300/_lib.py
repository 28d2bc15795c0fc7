"""ctypes binding of ``libshocks.so`` (the C ABI declared in ``include/shocks.h``).

There is no CPU fallback: every entry point needs the compiled library and a
CUDA device, and :func:`lib` raises if either is missing.
"""

from __future__ import annotations

import ctypes
import pathlib
import threading

import torch

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "libshocks.so"

SHK_OK = 0
SHK_EINVAL = 1
SHK_ENONFINITE = 2
SHK_ETIMEOUT = 3
SHK_ECUDA = 4
SHK_ENOMEM = 5
SHK_EUNSUPPORTED = 6
SHK_ETOOLARGE = 7

SHK_FLUX_RUSANOV, SHK_FLUX_LF, SHK_FLUX_ESWENO, SHK_FLUX_GODUNOV, SHK_FLUX_EO = 0, 1, 2, 3, 4
SHK_REC_WENOJS53, SHK_REC_ESWENO32, SHK_REC_LEARNED, SHK_REC_CONSTANT, SHK_REC_WENOJS32 = 0, 1, 2, 3, 4
SHK_REC_MUSCL, SHK_REC_MUSCLS = 5, 6
(SHK_LIM_NONE, SHK_LIM_MINMOD, SHK_LIM_MC, SHK_LIM_SUPERBEE, SHK_LIM_VANALBADA, SHK_LIM_VANLEER,
 SHK_LIM_KOREN) = range(7)
SHK_EQ_BURGERS, SHK_EQ_ADVECTION, SHK_EQ_LWR = 0, 1, 2
SHK_F64, SHK_F32 = 0, 1

# device status bits (csrc/device.cuh)
ERR_NONFINITE = 1
ERR_TIMEOUT = 2
ERR_BOUNDS = 4


class ShkScheme(ctypes.Structure):
    _fields_ = [
        ("flux", ctypes.c_int32),
        ("rec", ctypes.c_int32),
        ("equation", ctypes.c_int32),
        ("limiter", ctypes.c_int32),
        ("eps", ctypes.c_double),
        ("delta", ctypes.c_double),
        ("nu", ctypes.c_double),
        ("speed", ctypes.c_double),
        ("mlp", ctypes.c_void_p),
        ("tau", ctypes.c_float),
        ("band", ctypes.c_float),
        ("dev", ctypes.c_float),
        ("norm_eps", ctypes.c_float),
    ]


SHK_BC_PERIODIC, SHK_BC_DIRICHLET, SHK_BC_NEUMANN = 0, 1, 2


class ShkBoundary(ctypes.Structure):
    _fields_ = [
        ("left", ctypes.c_int32),
        ("right", ctypes.c_int32),
        ("dirichlet", ctypes.c_double * 18),  # [stage][side][k]
        ("neumann", ctypes.c_double * 6),     # [stage][side]
    ]


class ShkPlanOpts(ctypes.Structure):
    _fields_ = [
        ("dtype", ctypes.c_int32),
        ("tile", ctypes.c_int32),
        ("max_steps", ctypes.c_int32),
        ("ctas_per_sm", ctypes.c_int32),
    ]


_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double
_SCH = ctypes.POINTER(ShkScheme)

# name -> (restype, argtypes)
SIGNATURES: dict[str, tuple] = {
    "shk_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "shk_version": (ctypes.c_int, []),
    "shk_max_wavespeed_f64": (ctypes.c_int, [_SCH, _P, _I64, _I32, _P, _P]),
    "shk_apply_operator_f64": (ctypes.c_int, [_SCH, _P, _P, _I64, _I32, _D, _P, _P]),
    "shk_predict_timestep_f64": (ctypes.c_int, [_SCH, _P, _I64, _I32, _D, _D, _P, _P]),
    "shk_ssprk33_step_f64": (ctypes.c_int, [_SCH, _P, _P, _I64, _I32, _D, _D, _P]),
    "shk_apply_operator_bc_f64": (ctypes.c_int, [_SCH, ctypes.POINTER(ShkBoundary), _P, _P, _I64,
                                                 _I32, _D, _P, _P]),
    "shk_ssprk33_step_bc_f64": (ctypes.c_int, [_SCH, ctypes.POINTER(ShkBoundary), _P, _P, _I64,
                                               _I32, _D, _D, _P]),
    "shk_plan_create": (
        ctypes.c_int,
        [_SCH, _I32, _P, _P, _P, _D, ctypes.POINTER(ShkPlanOpts), ctypes.POINTER(_P)],
    ),
    "shk_plan_destroy": (ctypes.c_int, [_P]),
    "shk_plan_reset": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "shk_plan_step": (ctypes.c_int, [_P, _P, _P, _I32, _P]),
    "shk_plan_step_graph": (ctypes.c_int, [_P, _P, _P, _I32, _P]),
    "shk_plan_set_fixed_dt": (ctypes.c_int, [_P, _P, _I32, _P]),
    "shk_plan_set_boundary": (ctypes.c_int, [_P, _I32, _I32, _P, _P, _P]),
    "shk_plan_set_boundary_steps": (ctypes.c_int, [_P, _I32, _I32, _P, _P, _I32, _P]),
    "shk_plan_state": (ctypes.c_int, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "shk_plan_copy_time": (ctypes.c_int, [_P, _P, _P]),
    "shk_plan_copy_dt_history": (ctypes.c_int, [_P, _P, _P]),
    "shk_plan_status": (ctypes.c_int, [_P, ctypes.POINTER(_I32), _P]),
    "shk_plan_reduce": (ctypes.c_int, [_P, _P, _I32, _P, _P]),
    "shk_host_stepper_create": (
        ctypes.c_int,
        [_SCH, _I32, _P, _P, _P, _D, ctypes.POINTER(ShkPlanOpts), _I32, ctypes.POINTER(_P)],
    ),
    "shk_host_stepper_destroy": (ctypes.c_int, [_P]),
    "shk_host_stepper_num_chunks": (ctypes.c_int, [_P]),
    "shk_host_stepper_advance": (ctypes.c_int, [_P, _P, _P, _I32, _P]),
    "shk_host_stepper_status": (ctypes.c_int, [_P, ctypes.POINTER(_I32), _P]),
    "shk_host_stepper_set_boundary": (ctypes.c_int, [_P, _I32, _I32, _P, _P, _P]),
    "shk_ssprk33_vjp_f64": (ctypes.c_int, [_SCH, _P, _P, _P, _I64, _I32, _D, _D, _P]),
    "shk_ssprk33_vjp_bc_f64": (ctypes.c_int, [_SCH, ctypes.POINTER(ShkBoundary), _P, _P, _P, _I64,
                                              _I32, _D, _D, _P]),
    "shk_plan_forward_checkpointed": (ctypes.c_int, [_P, _P, _P, _I32, _P, _I32, _P]),
    "shk_plan_adjoint": (ctypes.c_int, [_P, _P, _I32, _I32, _P, _P, _P, _P]),
    "shk_plan_adjoint_stage_bytes": (ctypes.c_int, [_P, ctypes.POINTER(_I64)]),
    "shk_plan_adjoint_staged": (ctypes.c_int, [_P, _P, _I32, _I32, _P, _P, _P, _P, _P]),
    "shk_ghosted_workspace_bytes": (ctypes.c_int64, [_I64, _I32]),
    "shk_apply_operator_ghosted_f64": (ctypes.c_int, [_SCH, ctypes.POINTER(ShkBoundary), _P, _P, _I64,
                                                      _I32, _D, _P, _I64, _P]),
    "shk_ssprk33_step_ghosted_f64": (ctypes.c_int, [_SCH, ctypes.POINTER(ShkBoundary), _P, _P, _I64,
                                                    _I32, _D, _D, _P, _I64, _P]),
    "shk_ssprk33_vjp_ghosted_f64": (ctypes.c_int, [_SCH, ctypes.POINTER(ShkBoundary), _P, _P, _P, _I64,
                                                   _I32, _D, _D, _P, _I64, _P]),
    "shk_apply_operator_lf_noalloc_f64": (ctypes.c_int, [_SCH, _P, _P, _I64, _I32, _D, _P]),
    "shk_apply_operator_lf_noalloc_max_cells": (ctypes.c_int64, []),
    "shk_mlp_num_params": (ctypes.c_int, []),
    "shk_mlp_workspace_bytes": (ctypes.c_int64, [_I64]),
    "shk_mlp_loss_grad_f32": (ctypes.c_int, [_P, _P, _P, _P, _I64, ctypes.c_float, ctypes.c_float,
                                             _P, _P, _P, _I64, _P]),
    "shk_mlp_adam_f32": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_float, ctypes.c_float,
                                        ctypes.c_float, ctypes.c_float, _I32, _P]),
    "shk_learned_faces_f32": (ctypes.c_int, [_SCH, _P, _P, _I64, _P]),
    "shk_measure_fp_peak": (ctypes.c_int, [_I32, _I32, ctypes.POINTER(_D)]),
}

# prototypes of the bounds-check build's two extra entry points (include/shocks_check.h)
CHECK_SIGNATURES: dict[str, tuple] = {
    "shk_check_bounds": (ctypes.c_int, [_I32, _P, _P, _P, _P, _P]),
    "shk_check_force_timeout": (ctypes.c_int, [ctypes.c_uint32, _I64]),
}
CHECK_LIB_PATH = HERE / "libshocks_check.so"

_lock = threading.Lock()
_lib = None


class ShocksError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = errstr(status)
        super().__init__(f"{what}: {msg} (status {status})" if what else msg)


def errstr(status: int) -> str:
    names = {
        SHK_OK: "ok",
        SHK_EINVAL: "invalid argument",
        SHK_ENONFINITE: "Time step is not finite",
        SHK_ETIMEOUT: "bounded device wait expired",
        SHK_ECUDA: "CUDA runtime error",
        SHK_ENOMEM: "out of device memory",
        SHK_EUNSUPPORTED: "unsupported scheme combination",
        SHK_ETOOLARGE: "size exceeds the static scratch of the no-allocation entry point",
    }
    return names.get(status, f"unknown status {status}")


def load_library(path: pathlib.Path | None = None) -> ctypes.CDLL:
    """Load ``libshocks.so`` and declare its prototypes (no CUDA call is made)."""
    path = pathlib.Path(path or LIB_PATH)
    if not path.exists():
        raise ImportError(
            f"{path} is missing: build it with `python -m pyshocks_gb300._build` "
            "(or __graft_entry__.build()); there is no CPU fallback"
        )
    cdll = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(cdll, name)
        fn.restype = res
        fn.argtypes = args
    return cdll


def load_check_library() -> ctypes.CDLL:
    """Load the bounds-check build ``libshocks_check.so`` (the library's ABI plus
    ``shk_check_bounds`` and ``shk_check_force_timeout``); a test instrument,
    never loaded by the package itself."""
    cdll = load_library(CHECK_LIB_PATH)
    for name, (res, args) in CHECK_SIGNATURES.items():
        fn = getattr(cdll, name)
        fn.restype = res
        fn.argtypes = args
    return cdll


def lib() -> ctypes.CDLL:
    """The loaded library; raises if it is not built or no CUDA device exists."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not torch.cuda.is_available():
                    raise RuntimeError(
                        "pyshocks_gb300 needs a CUDA device (GB300); there is no CPU fallback"
                    )
                _lib = load_library()
    return _lib


def check(status: int, what: str = "") -> None:
    if status != SHK_OK:
        if status == SHK_ENONFINITE:
            raise ValueError(f"Time step is not finite ({what})")
        raise ShocksError(status, what)


def stream_handle(stream: torch.cuda.Stream | None = None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else int(t.data_ptr())
