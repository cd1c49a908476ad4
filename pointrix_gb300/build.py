"""Builds ``libpointrix_gb300.so`` from ``csrc/*.cu`` with nvcc for sm_103a.

The library has no torch headers in it (plain C ABI), so each translation
unit compiles in seconds; units are compiled in parallel and linked with the
static CUDA runtime.  ``project.cu`` is compiled with ``-fmad=false`` so that
its integer outputs are reproducible by an IEEE float32 CPU rendition.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB_NAME = "libpointrix_gb300.so"
LIB_PATH = PKG / LIB_NAME
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
NO_FMA = {"project.cu"}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pointrix_gb300")
    return cand


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _compile(src: Path, out: Path, extra: list[str]) -> None:
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(out)]
    if src.name in NO_FMA:
        cmd.insert(-4, "-fmad=false")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile every ``csrc/*.cu`` and link ``libpointrix_gb300.so`` in the
    package directory; skipped when the library is newer than all sources."""
    srcs = sources()
    deps = srcs + sorted(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "pointrix_gb300.h"]
    if (not force and LIB_PATH.exists()
            and LIB_PATH.stat().st_mtime > max(p.stat().st_mtime for p in deps)):
        return LIB_PATH
    bdir = PKG / "_build"
    bdir.mkdir(exist_ok=True)
    objs = [bdir / (s.stem + ".o") for s in srcs]
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], extra or []), zip(srcs, objs)))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    if verbose:
        print(f"built {LIB_PATH}", file=sys.stderr)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
