"""Build the CPU oracle (test infrastructure only).

Compiles oracle/umt_oracle.cpp into oracle/_build/liboracle_umt.so with
floating-point contraction disabled so that the restated Fortran arithmetic
keeps its operation order on both x86-64 and aarch64 hosts.

When the UMT source tree is present on this machine (it is not on the GPU
hosts), also builds the pieces of the reference that compile on their own
into oracle/_ref/ (see oracle/ref_build.py).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle_umt.so")


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "umt_oracle.cpp")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(src)):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", src, "-o", LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
