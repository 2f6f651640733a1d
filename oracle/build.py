"""Build recipe of the CPU oracle (test infrastructure only).

Compiles ``pm_oracle.c`` with gcc into ``oracle/_build/libpmoracle.so``:
IEEE f32 (``-ffp-contract=off``, no fast-math) so its arithmetic is the
reference kernels' operation order exactly, OpenMP for the loops the
reference runs in parallel. Portable C: builds the same on x86-64 and aarch64.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "pm_oracle.c"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libpmoracle.so"
CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
          "-fno-unsafe-math-optimizations"]


def build(force: bool = False) -> Path:
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler found to build the oracle")
    tmp = LIB.with_suffix(".so.tmp")
    r = subprocess.run([cc, *CFLAGS, str(SRC), "-o", str(tmp), "-lm"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":  # pragma: no cover
    print(build(force=True))
