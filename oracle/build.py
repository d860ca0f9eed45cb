"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/pdipc_oracle.cpp into oracle/liborc.so with g++ and OpenMP.
-ffp-contract=off keeps the arithmetic identical on x86 and Arm hosts.
The reference's project cannot be built here (MSVC; Eigen, Qt, oneTBB and
BVH_lib are absent), but its PD-IPC kernels can: oracle/build_ref.py compiles
them for the host into oracle/_ref, and they pin this restatement
(tests/golden/ref_kernels.npz).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "pdipc_oracle.cpp")
OUT = os.path.join(HERE, "liborc.so")


def build(force: bool = False) -> str:
    if (not force and os.path.exists(OUT)
            and os.path.getmtime(OUT) >= os.path.getmtime(SRC)
            and os.path.getmtime(OUT) >= os.path.getmtime(os.path.join(ROOT, "include", "pdipc.h"))):
        return OUT
    cmd = ["g++", "-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-I" + os.path.join(ROOT, "include"), SRC, "-o", OUT + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
