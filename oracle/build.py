"""Build recipe for the CPU checkers (test infrastructure only).

1. oracle/libpa_oracle.so  <- oracle/pa_oracle.c (the project's plain-C
   restatement), gcc.
2. oracle/_ref/libpa_ref.so <- the reference's own headers, compiled
   unchanged with oracle/ref_capi.cpp, the TBB stand-in (oracle/tbb_shim) and
   the Copy.h stand-in (oracle/ref_stub), g++.

The reference headers are read from the reference checkout: the directory
named by the environment variable PA_REFERENCE_DIR, else `reference` beside
this repository's root.  The include closure of ref_capi.cpp is also staged
(unmodified, never committed: oracle/_ref/ is git-ignored) in
oracle/_ref/src/, so that a machine without the checkout (such as an aarch64
host, on which x86 objects cannot run) rebuilds the same reference code from
there.  Nothing here is run by the product path.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
REF_OUT = ORACLE / "_ref"
REF_SRC_STAGE = REF_OUT / "src"
REFERENCE = Path(os.environ.get("PA_REFERENCE_DIR", str(ORACLE.parent.parent / "reference")))

ORACLE_LIB = ORACLE / "libpa_oracle.so"
REF_LIB = REF_OUT / "libpa_ref.so"

_INCLUDE_RE = re.compile(r'^\s*#\s*include\s*"([^"]+)"', re.M)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _newer(out: Path, *inputs: Path) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in inputs if p.exists())


def build_oracle(force: bool = False) -> Path:
    src = ORACLE / "pa_oracle.c"
    if force or not _newer(ORACLE_LIB, src, Path(__file__)):
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-Wall", str(src), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def _closure(root_files: list[Path], search: list[Path]) -> set[str]:
    """Names of the reference headers reachable from root_files."""
    seen: set[str] = set()
    todo = list(root_files)
    while todo:
        f = todo.pop()
        for name in _INCLUDE_RE.findall(f.read_text(errors="replace")):
            if name in seen:
                continue
            for d in search:
                if (d / name).exists():
                    if d == REFERENCE or d == REF_SRC_STAGE:
                        seen.add(name)
                        todo.append(d / name)
                    break
    return seen


def _stage_reference() -> Path | None:
    """Returns the directory to compile the reference from, staging it when
    the reference checkout is available."""
    if REFERENCE.is_dir():
        names = _closure([ORACLE / "ref_capi.cpp"], [ORACLE / "ref_stub", REFERENCE])
        REF_SRC_STAGE.mkdir(parents=True, exist_ok=True)
        for n in sorted(names):
            dst = REF_SRC_STAGE / n
            if not dst.exists() or dst.stat().st_mtime < (REFERENCE / n).stat().st_mtime:
                shutil.copy2(REFERENCE / n, dst)
        return REFERENCE
    if REF_SRC_STAGE.is_dir() and any(REF_SRC_STAGE.iterdir()):
        return REF_SRC_STAGE
    return None


def build_ref(force: bool = False) -> Path | None:
    """Builds oracle/_ref/libpa_ref.so; None if the reference sources are
    not available on this machine."""
    src_dir = _stage_reference()
    if src_dir is None:
        return None
    REF_OUT.mkdir(exist_ok=True)
    capi = ORACLE / "ref_capi.cpp"
    deps = [capi, ORACLE / "tbb_shim" / "tbb" / "tbb.h", ORACLE / "ref_stub" / "Copy.h", Path(__file__)]
    if force or not _newer(REF_LIB, *deps):
        _run(["g++", "-std=c++20", "-O3", "-fPIC", "-shared", "-pthread", "-include", "cstring",
              "-D_GLIBCXX_USE_TBB_PAR_BACKEND=0", f"-I{ORACLE / 'tbb_shim'}", f"-I{ORACLE / 'ref_stub'}",
              f"-I{src_dir}", str(capi), "-o", str(REF_LIB)])
    return REF_LIB


def build_all(force: bool = False) -> None:
    build_oracle(force)
    build_ref(force)


if __name__ == "__main__":
    import sys
    build_all(force="--force" in sys.argv)
    print(ORACLE_LIB, REF_LIB if REF_LIB.exists() else "(reference not built)")
