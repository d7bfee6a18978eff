"""Build recipe for the reference-side checkers (test infrastructure).

Reads the reference tree named by the environment variable IDB_REFERENCE_TREE
(required; nothing is built without it) and writes only into oracle/_ref/:

* ``ref_eps``: oracle/ref_eps_harness.cpp compiled with g++ against the
  reference's own cuda/SpecialFunctors.hcu (the threshold functor).
* ``ref_dbscan``: the reference's clustering translation unit, cuda/Interlink.cu
  with every header of the reference it includes, compiled with g++ on the host
  execution model of oracle/ref_emu.h and linked with
  oracle/ref_dbscan_harness.cpp.  The sources are streamed from where they lie
  into the compiler (``#line`` markers keep their file names and line numbers);
  the one change on the way is the kernel-launch syntax ``k<<<g, b, s>>>(a);``,
  which g++ cannot parse and which becomes
  ``::emu::launch("k", ::emu::Config(g, b, s), [&]() { k(a); });``.
  Thrust runs on its CPP (host) backend.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
EPS_EXE = os.path.join(OUT_DIR, "ref_eps")
DBSCAN_EXE = os.path.join(OUT_DIR, "ref_dbscan")
CUDA_INC = "/usr/local/cuda/include"

_INCLUDE = re.compile(r'^\s*#\s*include\s+"([^"]+)"')
_LAUNCH = re.compile(r'(\b\w+)\s*<<<(.*?)>>>\s*\((.*?)\)\s*;', re.S)


def reference_tree() -> str:
    """The reference tree, or '' when IDB_REFERENCE_TREE does not name one."""
    ref = os.environ.get("IDB_REFERENCE_TREE", "")
    return ref if ref and os.path.isfile(os.path.join(ref, "cuda", "Interlink.cu")) else ""


def _launch(m: re.Match) -> str:
    name, cfg, args = m.group(1), m.group(2), m.group(3)
    return '::emu::launch("%s", ::emu::Config(%s), [&]() { %s(%s); });' % (name, cfg, name, args)


def _stream(path: str, seen: set, out: list) -> None:
    """Append `path` to `out` with its reference-local includes inlined once
    each (every reference header is include-once) and launches rewritten."""
    path = os.path.realpath(path)
    if path in seen:
        return
    seen.add(path)
    with open(path, encoding="latin-1") as f:
        text = _LAUNCH.sub(_launch, f.read())
    out.append('#line 1 "%s"\n' % path)
    for no, line in enumerate(text.split("\n"), 1):
        m = _INCLUDE.match(line)
        inc = os.path.join(os.path.dirname(path), m.group(1)) if m else ""
        if inc and os.path.isfile(inc):
            _stream(inc, seen, out)
            out.append('#line %d "%s"\n' % (no + 1, path))
        else:
            out.append(line + "\n")


def _newer(target: str, *deps: str) -> bool:
    return os.path.exists(target) and all(os.path.getmtime(target) >= os.path.getmtime(d)
                                          for d in deps)


def build_eps(ref: str, force: bool = False) -> str:
    src = os.path.join(HERE, "ref_eps_harness.cpp")
    if not force and _newer(EPS_EXE, src):
        return EPS_EXE
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-x", "c++",
           "-I" + os.path.join(ref, "cuda"), "-I" + os.path.join(CUDA_INC, "cccl"), "-I" + CUDA_INC,
           "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP", src, "-o", EPS_EXE]
    subprocess.run(cmd, check=True)
    return EPS_EXE


def build_dbscan(ref: str, force: bool = False) -> str:
    own = [os.path.join(HERE, f) for f in ("ref_emu.h", "ref_emu.cpp", "ref_dbscan_harness.cpp")]
    if not force and _newer(DBSCAN_EXE, *own, __file__):
        return DBSCAN_EXE
    os.makedirs(OUT_DIR, exist_ok=True)
    stream: list = []
    _stream(os.path.join(ref, "cuda", "Interlink.cu"), set(), stream)
    common = ["-std=c++17", "-O2", "-ffp-contract=off", "-w",
              "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP",
              "-I" + os.path.join(ref, "cuda"), "-I" + os.path.join(CUDA_INC, "cccl"),
              "-I" + CUDA_INC]
    obj = os.path.join(OUT_DIR, "interlink.o")
    subprocess.run(["g++", *common, "-include", os.path.join(HERE, "ref_emu.h"),
                    "-x", "c++", "-", "-c", "-o", obj],
                   input="".join(stream).encode("latin-1"), check=True)
    tmp = DBSCAN_EXE + ".tmp%d" % os.getpid()
    subprocess.run(["g++", *common, "-I" + HERE, own[1], own[2], obj, "-o", tmp], check=True)
    os.replace(tmp, DBSCAN_EXE)
    return DBSCAN_EXE


def build(force: bool = False) -> str:
    """Builds both checkers; returns the ref_dbscan path ('' without a tree)."""
    ref = reference_tree()
    if not ref:
        return ""
    build_eps(ref, force)
    return build_dbscan(ref, force)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv) or "IDB_REFERENCE_TREE does not name a reference tree")
