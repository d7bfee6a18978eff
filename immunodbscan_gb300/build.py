"""In-tree build of libimmunodbscan_gb300.so (sm_103a) and the psdbscan host.

nvcc compiles each translation unit of csrc/ in parallel for
``-gencode arch=compute_103a,code=sm_103a`` and links one shared library with
the C ABI of include/immunodbscan_gb300.h.  g++ builds the psdbscan command-line
host (host/) against that library.  Outputs go to immunodbscan_gb300/_build/.
Portable host flags only: the same recipe runs on x86_64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libimmunodbscan_gb300.so")
CLI = os.path.join(OUT, "psdbscan")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "immunodbscan_gb300.h"))
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + _headers()):
        return obj
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj + ".tmp"]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas and r.stderr:
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build_library(force: bool = False, verbose_ptxas: bool = False, jobs: int = 0) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = _sources()
    if force:
        for s in srcs:
            o = os.path.join(OUT, os.path.basename(s) + ".o")
            if os.path.exists(o):
                os.remove(o)
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def build_cli(force: bool = False) -> str:
    """psdbscan: the reference's command-line host, linked to the library."""
    if not os.path.isdir(HOST):
        return ""
    srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp"))
    hdrs = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".hpp")]
    if not srcs:
        return ""
    if not force and not _stale(CLI, srcs + hdrs + [LIB]):
        return CLI
    tmp = CLI + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-pthread", "-I" + INCLUDE, "-I" + HOST, *srcs, "-o", tmp,
           "-L" + OUT, "-limmunodbscan_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"psdbscan build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CLI)
    return CLI


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    lib = build_library(force=force, verbose_ptxas=verbose_ptxas)
    build_cli(force=force)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
