"""Build the oracle's C restatement (krylov_c.c) into
oracle/_build/liboracle_krylov.so.

TEST INFRASTRUCTURE ONLY: the library is the checker's iterative solver and
the benchmark's CPU baseline; the product never loads it.  Built with OpenMP
when the compiler supports it, otherwise single-threaded.

Usage: python oracle/build.py   (or build() of this module)
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle_krylov.so"
SRC = HERE / "krylov_c.c"


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    base = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-Wall", "-o", str(tmp), str(SRC), "-lm"]
    r = subprocess.run(base[:1] + ["-fopenmp"] + base[1:], capture_output=True, text=True)
    if r.returncode != 0:
        r = subprocess.run(base, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
