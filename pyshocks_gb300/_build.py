"""Build ``libshocks.so`` (all CUDA sources under ``csrc/``) for sm_103a, in tree.

Translation units compile in parallel; each gets exactly one ``-gencode``
(``arch=compute_103a,code=sm_103a``). IEEE division and square root stay on
(no fast-math): the FP64 path must reproduce the reference to round-off.
"""

from __future__ import annotations

import os
import pathlib
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
LIB = HERE / "libshocks.so"
BUILD = HERE / "_build"

GENCODE = "arch=compute_103a,code=sm_103a"


def nvcc_path() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libshocks")
    return cand


def sources() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*.cu"))


def _compile(nvcc: str, src: pathlib.Path, extra: list[str]) -> pathlib.Path:
    obj = BUILD / (src.stem + ".o")
    cmd = [
        nvcc, "-gencode", GENCODE, "-O3", "-lineinfo", "-std=c++17",
        "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-c",
        "-I", str(HERE.parent / "include"), *extra, "-o", str(obj), str(src),
    ]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(force: bool = False, extra: list[str] | None = None, verbose: bool = False) -> pathlib.Path:
    """Compile every ``csrc/*.cu`` and link ``libshocks.so``; returns its path."""
    srcs = sources()
    deps = srcs + sorted(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "shocks.h"]
    if LIB.exists() and not force:
        newest = max(p.stat().st_mtime for p in deps)
        if LIB.stat().st_mtime >= newest:
            return LIB
    nvcc = nvcc_path()
    BUILD.mkdir(exist_ok=True)
    extra = list(extra or [])
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, extra), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, "-gencode", GENCODE, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
