"""Build ``libshocks.so`` (all CUDA sources under ``csrc/``) for sm_103a, in tree.

Translation units compile in parallel; each gets exactly one ``-gencode``
(``arch=compute_103a,code=sm_103a``). IEEE division and square root stay on
(no fast-math): the FP64 path must reproduce the reference to round-off.

Two variants come from the same sources: ``libshocks.so`` (the library) and
``libshocks_check.so``, the bounds-check build (``-DSHOCKS_BOUNDS_CHECK``:
every window, stage-storage and state index checked, violations logged in a
device word; ``include/shocks_check.h``), which the tests use as the memory
checker of the kernels.
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


VARIANTS = {
    "lib": (LIB, BUILD, []),
    "check": (HERE / "libshocks_check.so", HERE / "_build_check", ["-DSHOCKS_BOUNDS_CHECK"]),
}


def _compile(nvcc: str, src: pathlib.Path, outdir: pathlib.Path, extra: list[str]) -> pathlib.Path:
    obj = outdir / (src.stem + ".o")
    cmd = [
        nvcc, "-gencode", GENCODE, "-O3", "-lineinfo", "-std=c++17",
        "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-c",
        "-I", str(HERE.parent / "include"), *extra, "-o", str(obj), str(src),
    ]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


def _stale(lib: pathlib.Path) -> bool:
    deps = sources() + sorted(CSRC.glob("*.cuh")) + sorted((HERE.parent / "include").glob("*.h"))
    return not lib.exists() or lib.stat().st_mtime < max(p.stat().st_mtime for p in deps)


def build(force: bool = False, extra: list[str] | None = None, verbose: bool = False,
          variants: tuple[str, ...] = ("lib",)) -> pathlib.Path:
    """Compile every ``csrc/*.cu`` and link the requested variants
    (``"lib"``: ``libshocks.so``, ``"check"``: ``libshocks_check.so``), all
    translation units in one parallel pool; returns the first variant's path."""
    todo = [v for v in variants if force or _stale(VARIANTS[v][0])]
    if not todo:
        return VARIANTS[variants[0]][0]
    nvcc = nvcc_path()
    srcs = sources()
    jobs = []
    for v in todo:
        outdir = VARIANTS[v][1]
        outdir.mkdir(exist_ok=True)
        jobs += [(v, src, outdir, VARIANTS[v][2] + list(extra or [])) for src in srcs]
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(lambda j: (j[0], _compile(nvcc, j[1], j[2], j[3])), jobs))
    for v in todo:
        lib = VARIANTS[v][0]
        tmp = lib.with_suffix(".so.tmp")
        cmd = [nvcc, "-gencode", GENCODE, "-shared", "-o", str(tmp),
               *[str(o) for vv, o in objs if vv == v]]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, lib)
        if verbose:
            print(f"built {lib}", file=sys.stderr)
    return VARIANTS[variants[0]][0]


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          variants=("lib", "check") if "--check" in sys.argv else ("lib",))
