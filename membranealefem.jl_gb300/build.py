"""Build libmafem.so in-tree for sm_103a (nvcc, one -gencode, parallel compiles).

Usage: python membranealefem.jl_gb300/build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmafem.so")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["mesh.cpp", "elem.cu", "assemble.cu", "band_lu.cu", "band_lu_blk.cu", "band_lu_persist.cu", "band_lu_patch.cu", "api.cu", "noalloc.cu", "state_io.cpp"]
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]


def _deps_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "mafem.h")]
    return max(os.path.getmtime(f) for f in files)


def _compile(src: str) -> str:
    out = os.path.join(OBJ, src + ".o")
    cmd = [NVCC, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", out]
    if src.endswith(".cpp"):
        cmd = [NVCC, *FLAGS, "-x", "c++", "-c", os.path.join(CSRC, src), "-o", out]
    subprocess.run(cmd, check=True)
    return out


def build(force: bool = False) -> str:
    """Compile every translation unit and link libmafem.so (skipped if up to date)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    subprocess.run([NVCC, *ARCH, "-shared", "--cudart", "shared", "-o", tmp, *objs], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
