"""CPU checks of the C-ABI boundary: the library builds, loads without a GPU and
exports every function ``include/*.h`` declares, with matching ctypes
prototypes. No compute call is made here."""

from __future__ import annotations

import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _declared_functions(header: str = "shocks.h") -> list[str]:
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(shk_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def cdll():
    from pyshocks_gb300 import _build, _lib

    _build.build()
    return _lib.load_library()


@pytest.fixture(scope="module")
def checked_cdll():
    from pyshocks_gb300 import _build, _lib

    _build.build(variants=("check",))
    return _lib.load_check_library()


def test_header_declares_functions():
    names = _declared_functions()
    assert "shk_apply_operator_f64" in names
    assert "shk_plan_step" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(cdll):
    missing = [n for n in _declared_functions() if not hasattr(cdll, n)]
    assert not missing, missing


def test_ctypes_prototypes_cover_header(cdll):
    from pyshocks_gb300 import _lib

    assert set(_declared_functions()) == set(_lib.SIGNATURES), (
        set(_declared_functions()) ^ set(_lib.SIGNATURES))
    assert set(_declared_functions("shocks_check.h")) == set(_lib.CHECK_SIGNATURES)


def test_headers_cover_every_header_file():
    """Every header under include/ is one of the two checked here."""
    assert sorted(p.name for p in (ROOT / "include").glob("*.h")) == ["shocks.h", "shocks_check.h"]


def test_check_library_exports_the_library_abi_and_its_hooks(checked_cdll, cdll):
    """libshocks_check.so (the bounds-check build) is a drop-in for
    libshocks.so with two more entry points; libshocks.so has neither."""
    names = _declared_functions() + _declared_functions("shocks_check.h")
    missing = [n for n in names if not hasattr(checked_cdll, n)]
    assert not missing, missing
    for n in _declared_functions("shocks_check.h"):
        assert not hasattr(cdll, n), n


def test_strerror_without_gpu(cdll):
    # host-only entry point: safe without a device
    assert cdll.shk_strerror(2) == b"Time step is not finite"
    assert cdll.shk_version() >= 1


def test_invalid_arguments_rejected_on_host(cdll):
    """Argument validation happens before any CUDA call."""
    from pyshocks_gb300 import _lib

    s = _lib.ShkScheme(flux=0, rec=0, equation=0, eps=1e-6, delta=0.0, nu=1.0, speed=1.0)
    assert cdll.shk_apply_operator_f64(s, None, None, 256, 3, 0.1, None, None) == _lib.SHK_EINVAL
    bad = _lib.ShkScheme(flux=2, rec=0, equation=0)  # ES-WENO flux needs the ES-WENO rec
    assert cdll.shk_apply_operator_f64(bad, 8, 16, 256, 3, 0.1, None, None) == _lib.SHK_EINVAL
    assert cdll.shk_plan_step(None, None, None, 1, None) == _lib.SHK_EINVAL


def test_plan_arguments_rejected_on_host(cdll):
    """Empty batches, degenerate instances, bad cell sizes and tiles are refused
    before any device memory is touched (plans and host-buffer steppers)."""
    import ctypes

    import numpy as np

    from pyshocks_gb300 import _lib

    s = _lib.ShkScheme(flux=0, rec=0, equation=0, eps=1e-6, delta=0.0, nu=1.0, speed=1.0)
    out = ctypes.c_void_p()

    def create(offsets, dx, opts=None, *, chunks=None):
        off = np.asarray(offsets, dtype=np.int64)
        dxa = np.asarray(dx, dtype=np.float64)
        cfl = 0.5 * dxa
        B = len(off) - 1
        o = ctypes.byref(opts) if opts is not None else None
        if chunks is None:
            return cdll.shk_plan_create(s, B, off.ctypes.data, dxa.ctypes.data, cfl.ctypes.data,
                                        1.0, o, ctypes.byref(out))
        return cdll.shk_host_stepper_create(s, B, off.ctypes.data, dxa.ctypes.data,
                                            cfl.ctypes.data, 1.0, o, chunks, ctypes.byref(out))

    for chunks in (None, 4):
        assert create([0], [], chunks=chunks) == _lib.SHK_EINVAL  # no instance
        assert create([0, 2], [0.1], chunks=chunks) == _lib.SHK_EINVAL  # n < 3
        assert create([0, 64], [0.0], chunks=chunks) == _lib.SHK_EINVAL  # dx <= 0
        assert create([0, 64], [-0.1], chunks=chunks) == _lib.SHK_EINVAL
        for tile in (7, 8, 8200):  # not a multiple of 16 bytes, too short, too long
            opts = _lib.ShkPlanOpts(dtype=_lib.SHK_F64, tile=tile, max_steps=0, ctas_per_sm=0)
            assert create([0, 64], [0.1], opts, chunks=chunks) == _lib.SHK_EINVAL, tile
        opts = _lib.ShkPlanOpts(dtype=7, tile=0, max_steps=0, ctas_per_sm=0)
        assert create([0, 64], [0.1], opts, chunks=chunks) == _lib.SHK_EINVAL  # dtype
    # the learned reconstruction needs tiles of at least 512 cells
    s_learned = _lib.ShkScheme(flux=0, rec=_lib.SHK_REC_LEARNED, equation=0, eps=1e-6, delta=0.0,
                               nu=1.0, speed=1.0, mlp=1)
    off = np.array([0, 4096], dtype=np.int64)
    dxa = np.array([0.1])
    opts = _lib.ShkPlanOpts(dtype=_lib.SHK_F64, tile=256, max_steps=0, ctas_per_sm=0)
    assert cdll.shk_plan_create(s_learned, 1, off.ctypes.data, dxa.ctypes.data, dxa.ctypes.data,
                                1.0, ctypes.byref(opts), ctypes.byref(out)) == _lib.SHK_EINVAL
    assert out.value is None
    # host steppers step forward only and take a non-negative chunk count
    opts = _lib.ShkPlanOpts(dtype=_lib.SHK_F64, tile=0, max_steps=10, ctas_per_sm=0)
    assert create([0, 64], [0.1], opts, chunks=4) == _lib.SHK_EINVAL
    assert create([0, 64], [0.1], chunks=-1) == _lib.SHK_EINVAL
    assert cdll.shk_host_stepper_advance(None, None, None, 1, None) == _lib.SHK_EINVAL
    assert cdll.shk_host_stepper_num_chunks(None) == 0


def test_product_path_never_imports_the_oracle():
    """The package must not import, call or link anything under oracle/."""
    pkg = ROOT / "pyshocks_gb300"
    for p in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cuh")):
        text = p.read_text()
        assert "oracle" not in re.findall(r"(?:import|from)\s+(\w+)", text), p
        assert "numpy_ref" not in text and "torch_ref" not in text, p
