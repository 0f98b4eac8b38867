"""Builds the engine's shared library ``_wfs.so`` in-tree with nvcc for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel into ``_build/``
and linked into ``wavefunctionsimpython_gb300/_wfs.so`` (static cudart). Host
code is compiled with ``-ffp-contract=off`` so float32 geometry evaluated on
the host rounds the same way on x86_64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "_wfs.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-diag-suppress", "177", "-I", str(ROOT / "include")]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path("/usr/local/cuda/bin/nvcc")
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _deps_mtime():
    files = (list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h"))
             + list((ROOT / "include").glob("*.h")) + [Path(__file__)])
    return max(f.stat().st_mtime for f in files)


def _compile(src: Path, extra) -> Path:
    obj = BUILD / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> Path:
    """Compile and link ``_wfs.so``; skipped when it is newer than every source."""
    extra = list(extra_flags or [])
    if LIB.exists() and not force and LIB.stat().st_mtime >= _deps_mtime() and not extra:
        return LIB
    BUILD.mkdir(exist_ok=True)
    srcs = _sources()
    workers = min(len(srcs), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
