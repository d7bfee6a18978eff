"""Build recipe for the reference-side checker (test infrastructure).

Compiles oracle/ref_eps_harness.cpp with g++ against the reference's own
cuda/SpecialFunctors.hcu, where it lies in the reference tree, into
oracle/_ref/ref_eps.  Only the threshold functor compiles on a host: the rest
of the reference's path is CUDA kernels (shared memory, __syncthreads_count)
built with its CMake project and Boost, which is not done here.  Does nothing
when the reference tree is absent (the GPU machine).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("IDB_REFERENCE_TREE", "/root/reference")
OUT_DIR = os.path.join(HERE, "_ref")
EXE = os.path.join(OUT_DIR, "ref_eps")
CUDA_INC = "/usr/local/cuda/include"


def build(force: bool = False) -> str:
    hdr = os.path.join(REF, "cuda", "SpecialFunctors.hcu")
    src = os.path.join(HERE, "ref_eps_harness.cpp")
    if not os.path.exists(hdr):
        return ""
    if not force and os.path.exists(EXE) and os.path.getmtime(EXE) >= os.path.getmtime(src):
        return EXE
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-x", "c++",
           "-I" + os.path.join(REF, "cuda"), "-I" + os.path.join(CUDA_INC, "cccl"), "-I" + CUDA_INC,
           "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP", src, "-o", EXE]
    subprocess.run(cmd, check=True)
    return EXE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv) or "reference tree not present")
