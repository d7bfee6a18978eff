"""CPU-side checks: the kernels' integer helpers compiled as host code, the
C ABI library (loads, exports every declared symbol, reports a missing device),
and the Python mirror's argument handling."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "immunodbscan_gb300.h")


def test_bitops_host(tmp_path):
    exe = tmp_path / "test_bitops"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "immunodbscan_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "test_bitops.cpp"), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:idb_status|size_t|const char \*|int)\s+\*?(idb_\w+)\(",
                                 text, re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ["idb_cluster", "idb_cluster_device", "idb_batch_plan", "idb_batch_run",
              "idb_context_create", "idb_context_destroy", "idb_last_error"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    from immunodbscan_gb300 import _lib
    assert os.path.exists(_lib.LIB_PATH), "build the library first (__graft_entry__.build())"
    L = C.CDLL(_lib.LIB_PATH)
    for n in declared_functions():
        assert hasattr(L, n), f"{n} declared in the header but not exported"
    assert _lib.lib().idb_abi_version() == 1


def test_status_strings():
    from immunodbscan_gb300 import _lib
    for s in range(9):
        assert _lib.lib().idb_status_string(s)


def test_no_device_is_reported():
    """Without a GPU the library reports IDB_ERR_NO_DEVICE instead of crashing."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from immunodbscan_gb300 import IdbError, Context
    with pytest.raises(IdbError) as e:
        Context(0)
    assert e.value.status == 3


def test_interlink_rejects_bad_columns():
    from immunodbscan_gb300 import Interlink
    with pytest.raises(ValueError):
        Interlink([b"IGHV1*"], None, [b"CAR", b"CAK"], 2, [b"IGHV1*"], [], 0.1, 2, False)


def test_synthetic_workloads_shapes():
    from immunodbscan_gb300 import synth
    for k, scale in [(0, 0.1), (1, 0.01), (2, 0.002), (3, 0.002), (4, 0.0005)]:
        w = synth.workload(k, scale=scale)
        assert w.n == int(w.rep_off[-1])
        assert len(w.seq_off) == w.n + 1 and len(w.v_off) == w.n + 1
        L = w.lengths()
        assert L.min() >= 1
        if k == 1:
            assert np.all(L % 3 == 0)
    w = synth.workload(2, scale=0.002)
    assert w.n_rep == 64
