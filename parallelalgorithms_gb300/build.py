"""Builds the native library libpa_gb300.so in-tree.

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked into one
shared object next to this file.  nvcc cross-compiles without a GPU, so the
build runs on any machine with the CUDA 13 toolkit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libpa_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["pa_capi.cu", "pa_histogram.cu", "pa_onesweep.cu", "pa_sum.cu", "pa_select.cu", "pa_pipeline.cu",
                "pa_segmented.cu", "pa_noalloc.cu", "pa_serve.cu", "pa_partition.cu",
                "pa_inplace.cu"]
HOST_SOURCES = ["pa_workloads.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libpa_gb300.so")


def _sources() -> list[Path]:
    return [CSRC / s for s in CUDA_SOURCES + HOST_SOURCES if (CSRC / s).exists()]


def _compile(src: Path, extra: list[str]) -> Path:
    obj = BUILD / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
           f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj), *extra]
    if src.suffix == ".cpp":
        cmd = [nvcc(), "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O3", f"-I{INCLUDE}", f"-I{CSRC}",
               "-x", "c++", "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def _stale() -> bool:
    if not LIB.exists():
        return True
    newest = max(p.stat().st_mtime for p in list(CSRC.iterdir()) + [INCLUDE / "pa_gpu.h", Path(__file__)])
    flags = LIB.with_suffix(".flags")
    if (flags.read_text() if flags.exists() else "") != os.environ.get("PA_NVCC_FLAGS", ""):
        return True
    return LIB.stat().st_mtime < newest


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    """Compiles and links libpa_gb300.so unless it is up to date."""
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    # PA_NVCC_FLAGS: extra compiler flags (e.g. -D tuning switches of the kernels)
    extra += os.environ.get("PA_NVCC_FLAGS", "").split()
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt", "-ldl",
           "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    LIB.with_suffix(".flags").write_text(os.environ.get("PA_NVCC_FLAGS", ""))
    return LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build(force=force, verbose_ptxas="--ptxas-v" in sys.argv))
