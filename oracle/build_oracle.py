"""Build recipe for the CPU oracle (test infrastructure, see oracle.h).

Compiles oracle/oracle.cpp with g++ and OpenMP into oracle/_build/liboracle.so.
Portable flags only (the same recipe runs on x86_64 and aarch64 hosts).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.cpp")
    hdr = os.path.join(HERE, "oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared",
           "-fno-fast-math", "-ffp-contract=off", "-o", tmp, src]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
