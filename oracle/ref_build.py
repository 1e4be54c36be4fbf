"""Build the parts of the reference that compile on their own (test use only).

Outputs go to oracle/_ref/ (git-ignored):
  * libnbb.so        -- src/teton/misc/NormalizedBlackBody.cc, plain C++,
                        used to pin the oracle's black-body group integrals;
  * ref_sweep.cubin  -- device code of src/teton/gpu/GPU_SweepUCBxyz.cu for
                        sm_103a (kernels are extern "C"), launched by
                        tests/golden/gen_ref_sweep.py through the CUDA driver
                        API to produce golden sweep outputs.
The Fortran CPU path needs a Fortran compiler, MPI and Conduit, none of
which exist here, so it is not built.  Nothing is copied out of the source
tree; the compilers read the files where they lie.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# The UMT source tree: $UMT_REFERENCE, else a directory named "reference"
# beside this repository's checkout (absent on the GPU hosts).
REF = os.environ.get("UMT_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def build(force=False):
    src = os.path.join(REF, "src", "teton")
    if not os.path.isdir(src):
        return None
    os.makedirs(OUT, exist_ok=True)
    nbb = os.path.join(OUT, "libnbb.so")
    if force or not os.path.exists(nbb):
        subprocess.check_call(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                               os.path.join(src, "misc", "NormalizedBlackBody.cc"), "-o", nbb])
    cubin = os.path.join(OUT, "ref_sweep.cubin")
    if force or not os.path.exists(cubin):
        subprocess.check_call(["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                               "-I/usr/local/cuda/include/nvtx3",
                               os.path.join(src, "gpu", "GPU_SweepUCBxyz.cu"), "-o", cubin])
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
