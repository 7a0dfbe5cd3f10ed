"""Build libedgefem_gb300.so in-tree: the sm_103a kernels (nvcc) and the C++
host library (g++), linked against the CUDA runtime.

Usage: python edgefem_gb300/build.py   (or build() of this module)
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
OUT_DIR = PKG / "_build"
LIB = PKG / "libedgefem_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    return cu, cpp


def build(verbose: bool = False, force: bool = False) -> Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC), "-I", str(cuda / "include")]
    OUT_DIR.mkdir(exist_ok=True)
    cu, cpp = _sources()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.hpp")) + list((ROOT / "include").glob("*.h"))
    newest_header = max((h.stat().st_mtime for h in headers), default=0.0)
    jobs = []
    objs = []
    for src in cu + cpp:
        obj = OUT_DIR / (src.stem + (".cu.o" if src.suffix == ".cu" else ".o"))
        objs.append(obj)
        if (not force and obj.exists() and obj.stat().st_mtime >= src.stat().st_mtime
                and obj.stat().st_mtime >= newest_header):
            continue
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", *inc,
                   "-c", str(src), "-o", str(obj)]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-sign-compare", *inc,
                   "-c", str(src), "-o", str(obj)]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr, file=sys.stderr)
    relink = force or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs)
    if relink:
        tmp = LIB.with_suffix(".so.tmp")
        _run(["g++", "-shared", "-o", str(tmp), *map(str, objs), "-L", str(cuda / "lib64"),
              "-Wl,-rpath," + str(cuda / "lib64"), "-lcudart", "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
