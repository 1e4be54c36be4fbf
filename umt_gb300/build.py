"""Build libumt103.so (the C-ABI of include/umt103.h) for sm_103a, in-tree.

    python -m umt_gb300.build [--force]

Translation units are compiled in parallel with nvcc; geom_sched.cu is
compiled with -fmad=false so that geometry and dependency signs reproduce the
Fortran operation order exactly.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libumt103.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
UNITS = {
    "capi.cu": [],
    "geom_sched.cu": ["-fmad=false"],
    "sweep.cu": [],
    "sweep32.cu": [],
    "sweep32p.cu": [],
    "si.cu": [],
    "rz.cu": ["-Xcompiler", "-ffp-contract=off"],   # host-side RZ geometry, same rounding as the Fortran
    "noalloc.cu": [],
    "psib.cu": [],
    "learn.cu": [],
}


def _nvcc():
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if p and (os.path.exists(p) or p == "nvcc"):
            return p
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "umt103.h"))
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    nvcc = _nvcc()

    def comp(unit):
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OUT, unit.replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, *COMMON, *UNITS[unit], "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(len(UNITS)) as ex:
        results = list(ex.map(comp, UNITS))
    if verbose:
        for _, err in results:
            sys.stderr.write(err)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
