"""In-tree build of the CUDA library ``libgcpm.so`` for sm_103a.

The library is the hot path of this package; it is compiled by ``nvcc``
directly (one ``-gencode``, translation units in parallel, no CMake) and loaded
with ctypes by :mod:`galaxy_collision_gb300._native`. Object files go to
``_build/`` next to this file and the shared object beside the package sources,
both ignored by git.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR.parent / "csrc"
INCLUDE = PKG_DIR.parent.parent / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_PATH = PKG_DIR / "libgcpm.so"

SOURCES = ("ctx.cu", "multigrid.cu", "particles.cu", "sort.cu", "engine.cu", "noalloc.cu", "warmstart.cu", "viz.cu", "ic.cu")
ARCH_FLAGS = ("-gencode", "arch=compute_103a,code=sm_103a")
NVCC_FLAGS = ("-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2")


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgcpm.so")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile ``libgcpm.so`` (sm_103a) if any source is newer than it. Returns its path."""
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    headers = [CSRC / "common.cuh", CSRC / "umma.cuh", INCLUDE / "gcpm.h"]
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD_DIR / (Path(src).stem + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(s), "-o", str(o)]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout, r.stderr)

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB_PATH, objs):
        tmp = LIB_PATH.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH_FLAGS, "-shared", *map(str, objs), "-o", str(tmp)]
        run(cmd)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":  # pragma: no cover
    print(build(verbose=True))
