"""CPU checks of the C-ABI boundary: the library builds, loads without a GPU and
exports every function ``include/*.h`` declares, with matching ctypes
prototypes. No compute call is made here."""

from __future__ import annotations

import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _declared_functions() -> list[str]:
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(shk_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def cdll():
    from pyshocks_gb300 import _build, _lib

    _build.build()
    return _lib.load_library()


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


def test_product_path_never_imports_the_oracle():
    """The package must not import, call or link anything under oracle/."""
    pkg = ROOT / "pyshocks_gb300"
    for p in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cuh")):
        text = p.read_text()
        assert "oracle" not in re.findall(r"(?:import|from)\s+(\w+)", text), p
        assert "numpy_ref" not in text and "torch_ref" not in text, p
