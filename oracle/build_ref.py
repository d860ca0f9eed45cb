"""Build recipe for oracle/_ref: the reference's own PD-IPC kernels, run on the
host (test infrastructure only; it pins the oracle, nothing ships it).

The reference (lanlei/PD-IPC-ArmadilloDemo) is an MSVC/Qt project whose
build cannot run here, and its PD-IPC path exists only as CUDA kernels
(Simulator/PD-IPC/PdIpcGpuFunc.cu).  Those kernels are plain CUDA C, so this
recipe compiles them unmodified with the host C++ compiler under
oracle/cuda_emu.h, which runs a kernel's threads as fibers with real block
barriers.  Three things stand between the sources and g++, and each is
bridged in a generated build directory (oracle/_ref/gen, never committed):
  * include paths written with backslashes ("Simulator\\Cuda\\CudaHeader.cuh"):
    a forwarding header with that literal file name includes the real file
    from the reference tree;
  * CUDA, cuBLAS and thrust headers: empty stand-ins (the kernels use none of
    their declarations; cuda_emu.h provides dim3, the builtins and atomics);
  * the __host__ launch wrappers, written with <<< >>> launch syntax: the copy
    of PdIpcGpuFunc.cu in the build directory leaves every __host__ function
    definition out (declarations stay), and with them the two candidate-list
    kernels of the broad phase (getCcdPotentialICPairsListKernel,
    getDcdPotentialICPairsListKernel), which declare "int aId, int bId;", a
    form only the reference's MSVC-era front end accepts; the harness does not
    launch them.  Every other __global__ and __device__ function is copied
    byte for byte.  oracle/ref_harness.cpp launches the kernels in the order
    the reference's host code does.
Two builds: qeal = float (the reference's configuration, DataCore.h:8,19) and
qeal = double (the reference's own USE_DOUBLE_PRECISION switch).

The reference tree is read from $PDIPC_REFERENCE_DIR, default /root/reference.
Without it (for example on a machine that only runs the tests) nothing is
built and the committed golden fixtures stand in.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
GEN = os.path.join(OUT, "gen")
SHIM = os.path.join(GEN, "shim")

STUB_HEADERS = [
    "cuda_runtime.h", "device_launch_parameters.h", "cuda_runtime_api.h", "cuda.h", "cublas.h", "cublas_v2.h",
    "cusolverDn.h", "cusparse.h", "cusolverSp.h", "cusolverSp_LOWLEVEL_PREVIEW.h",
    "thrust/host_vector.h", "thrust/device_vector.h", "thrust/functional.h", "thrust/sort.h", "thrust/unique.h",
    "thrust/copy.h", "thrust/sequence.h", "thrust/count.h",
]
# backslash include names used by the kernel file and its header -> path in the tree
FORWARDS = {
    "Simulator\\Cuda\\CudaHeader.cuh": "Simulator/Cuda/CudaHeader.cuh",
    "Simulator\\Cuda\\CudaSVD.cu": "Simulator/Cuda/CudaSVD.cu",
    "Simulator\\Cuda\\CudaMatrixOperator.cu": "Simulator/Cuda/CudaMatrixOperator.cu",
}
KERNEL_FILE = "Simulator/PD-IPC/PdIpcGpuFunc.cu"
LEAVE_OUT = ("getCcdPotentialICPairsListKernel", "getDcdPotentialICPairsListKernel")
# variant -> (compiler defines, kernels also left out).  The tet kernel passes
# qeal* to float-only matrix helpers (PdIpcGpuFunc.cu:321,482), so it does not
# build with qeal = double in the reference either; the cloth path does.
VARIANTS = {"fp32": ([], ()), "fp64": (["-DUSE_DOUBLE_PRECISION"], ("solveVolumetricStrainConstraintKernel",))}


def reference_dir() -> str | None:
    d = os.environ.get("PDIPC_REFERENCE_DIR", "/root/reference")
    return d if os.path.exists(os.path.join(d, KERNEL_FILE)) else None


def lib_path(variant: str) -> str:
    return os.path.join(OUT, f"libpdipc_ref_{variant}.so")


def _skip_comment_or_literal(s: str, i: int) -> int:
    """If s[i] starts a comment or a string/char literal, the index past it; else i."""
    if s.startswith("//", i):
        j = s.find("\n", i)
        return len(s) if j < 0 else j
    if s.startswith("/*", i):
        j = s.find("*/", i + 2)
        return len(s) if j < 0 else j + 2
    if s[i] in "\"'":
        q, j = s[i], i + 1
        while j < len(s) and s[j] != q:
            j += 2 if s[j] == "\\" else 1
        return j + 1
    return i


def _leaves_out(src: str, i: int, leave_out: tuple) -> bool:
    """Does a function definition to leave out start at src[i]?"""
    if src.startswith("__host__", i):
        return True
    if src.startswith("__global__", i):
        head = src[i:i + 200].split("(", 1)[0].split()
        return len(head) >= 3 and head[2] in leave_out
    return False


def strip_host_definitions(src: str, leave_out: tuple = LEAVE_OUT) -> tuple[str, int]:
    """src without its __host__ function definitions and the kernels named in
    leave_out (from the keyword through the matching closing brace);
    declarations and every other byte are kept."""
    out, i, n, removed = [], 0, len(src), 0
    while i < n:
        j = _skip_comment_or_literal(src, i)
        if j != i:
            out.append(src[i:j])
            i = j
            continue
        if _leaves_out(src, i, leave_out) and (i == 0 or not (src[i - 1].isalnum() or src[i - 1] == "_")):
            # find '{' (a definition) or ';' (a declaration) at parenthesis depth 0
            k, depth = i, 0
            while k < n:
                k2 = _skip_comment_or_literal(src, k)
                if k2 != k:
                    k = k2
                    continue
                c = src[k]
                if c == "(":
                    depth += 1
                elif c == ")":
                    depth -= 1
                elif depth == 0 and c in "{;":
                    break
                k += 1
            if k < n and src[k] == "{":
                braces = 0
                while k < n:
                    k2 = _skip_comment_or_literal(src, k)
                    if k2 != k:
                        k = k2
                        continue
                    if src[k] == "{":
                        braces += 1
                    elif src[k] == "}":
                        braces -= 1
                        if braces == 0:
                            break
                    k += 1
                out.append("/* left out of the host build (oracle/build_ref.py) */")
                i = k + 1
                removed += 1
                continue
        out.append(src[i])
        i += 1
    return "".join(out), removed


def generate(ref: str) -> None:
    os.makedirs(os.path.join(SHIM, "thrust"), exist_ok=True)
    for h in STUB_HEADERS:
        with open(os.path.join(SHIM, h), "w") as f:
            f.write("/* stand-in: the kernels use nothing declared here (oracle/build_ref.py) */\n")
            if h in ("thrust/device_vector.h", "thrust/host_vector.h"):
                # named by the host wrappers' declarations in PdIpcGpuFunc.cuh
                f.write("#pragma once\nnamespace thrust { template <class T, class A = void> class device_vector; "
                        "template <class T, class A = void> class host_vector; }\n")
    for name, rel in FORWARDS.items():
        with open(os.path.join(SHIM, name), "w") as f:
            f.write(f'#include "{os.path.join(ref, rel)}"\n')
    with open(os.path.join(ref, KERNEL_FILE), encoding="utf-8", errors="replace") as f:
        src = f.read()
    for v, (_, extra) in VARIANTS.items():
        stripped, removed = strip_host_definitions(src, LEAVE_OUT + extra)
        if removed < 20:
            raise RuntimeError(f"expected the reference's __host__ wrappers in {KERNEL_FILE}, removed {removed}")
        os.makedirs(os.path.join(GEN, v), exist_ok=True)
        with open(os.path.join(GEN, v, "PdIpcGpuFunc_kernels.cu"), "w") as f:
            f.write(stripped)


def build(force: bool = False) -> dict[str, str] | None:
    ref = reference_dir()
    if ref is None:
        return None
    harness = os.path.join(HERE, "ref_harness.cpp")
    emu = os.path.join(HERE, "cuda_emu.h")
    srcs = [harness, emu, os.path.join(ref, KERNEL_FILE), __file__]
    libs = {}
    fresh = not force and all(
        os.path.exists(lib_path(v)) and all(os.path.getmtime(lib_path(v)) >= os.path.getmtime(s) for s in srcs)
        for v in VARIANTS)
    if not fresh:
        generate(ref)
    for v, (defs, _) in VARIANTS.items():
        out = lib_path(v)
        libs[v] = out
        if fresh:
            continue
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w", *defs,
               "-include", emu, "-I", SHIM, "-I", os.path.join(GEN, v), "-I", ref,
               "-I", os.path.join(ref, "Simulator", "PD-IPC"),
               harness, "-o", out + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference kernel build ({v}) failed:\n{r.stderr[-6000:]}")
        os.replace(out + ".tmp", out)
    return libs


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
