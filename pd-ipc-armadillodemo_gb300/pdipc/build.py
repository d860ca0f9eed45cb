"""Build recipe for libpdipc.so (sm_103a only).

Each translation unit is compiled by nvcc in parallel, then linked into
pd-ipc-armadillodemo_gb300/libpdipc.so with the CUDA runtime linked
statically.  No CMake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "libpdipc.so")
OBJ = os.path.join(PKG, "_build")

SOURCES = ["pd_kernels.cu", "pd_persistent.cu", "pd_persistent_band.cu", "collision_kernels.cu", "penalty_kernels.cu", "primitives.cu",
           "adjoint_kernels.cu", "solver.cu",
           "host_tables.cpp", "capi.cpp", "scene_io.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code must not fuse multiply-adds: the patch grid is computed in FP32 exactly as
# the reference does, and an Arm host compiler contracts a*b+c by default
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I" + INC, "-I" + CSRC]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(INC, "pdipc.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra: list[str]) -> str:
    s = os.path.join(CSRC, src)
    o = os.path.join(OBJ, src + ".o")
    if _stale(o, s):
        lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
        cmd = [nvcc()] + ARCH + COMMON + extra + lang + ["-c", s, "-o", o + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        os.replace(o + ".tmp", o)
    return o


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    if force:
        for f in os.listdir(OBJ):
            os.remove(os.path.join(OBJ, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if force or not os.path.exists(OUT) or any(os.path.getmtime(o) > os.path.getmtime(OUT) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", OUT + ".tmp"] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
