"""idb_dedupe_noalloc: duplicate collapse for callers that cannot allocate.

Some users of this library cannot call cudaMalloc: their device memory is owned
by another allocator, or they run in a loop where the device-wide
synchronisation of cudaMalloc/cudaFree is not allowed.  idb_dedupe_noalloc gives
them the duplicate-collapse step with its scratch in a fixed array inside the
library.  This test calls it through the C ABI on device columns and checks its
copies column against the one idb_cluster (the existing entry point) returns for
the same rows -- bit-exact, like every integer result in these tests -- on two
calls in a row with different inputs, so a call that left stale scratch behind
would fail the second comparison.  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from immunodbscan_gb300 import _lib, cluster_workload, synth

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 18


def _device(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host_bits(calls_blob, calls_off, genes):
    """uint64 bitsets (bit g = gene g is a substring of the call), one word."""
    n = len(calls_off) - 1
    out = np.zeros(n, np.uint64)
    blob = calls_blob.tobytes()
    for i in range(n):
        c = blob[calls_off[i]:calls_off[i + 1]]
        b = 0
        for g, name in enumerate(genes):
            if name and name in c:
                b |= 1 << g
        out[i] = b
    return out


def _noalloc(w, vbits=None):
    import torch
    seq = _device(w.seq_blob)
    off = _device(w.seq_off)
    rep = torch.zeros(w.n, dtype=torch.int32, device="cuda")
    cop = torch.zeros(w.n, dtype=torch.int32, device="cuda")
    vb = _device(vbits) if vbits is not None else None
    torch.cuda.synchronize()
    st = _lib.lib().idb_dedupe_noalloc(seq.data_ptr(), off.data_ptr(),
                                       vb.data_ptr() if vb is not None else None,
                                       1 if vb is not None else 0, None, 0, w.n,
                                       rep.data_ptr(), cop.data_ptr(), None)
    _lib.check(st)
    return rep.cpu().numpy().view(np.uint32), cop.cpu().numpy().view(np.uint32)


def _expected_reps(w, vbits=None):
    first = {}
    reps = np.zeros(w.n, np.uint32)
    for i in range(w.n):
        key = (w.seq(i), int(vbits[i]) if vbits is not None else 0)
        reps[i] = first.setdefault(key, i)
    return reps


def test_noalloc_matches_cluster_copies_twice():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    workloads = [synth.workload(0, scale=1.0), synth.workload(3, scale=0.05)]
    assert all(w.n <= MAX_ROWS for w in workloads)
    for w in workloads:                      # two calls in a row, different inputs
        rep, copies = _noalloc(w)
        ref = cluster_workload(w, None, no_v=True, no_j=True)
        assert np.array_equal(copies, ref.copies)
        assert np.array_equal(rep, _expected_reps(w))


def test_noalloc_with_v_bitsets():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    w = synth.workload(0, scale=0.5)
    vbits = _host_bits(w.v_blob, w.v_off, w.v_genes)
    rep, copies = _noalloc(w, vbits)
    ref = cluster_workload(w, None, no_j=True)
    assert np.array_equal(copies, ref.copies)
    assert np.array_equal(rep, _expected_reps(w, vbits))


def test_noalloc_rejects_oversized_input():
    dummy = C.c_uint32()
    p = C.cast(C.pointer(dummy), C.c_void_p)
    st = _lib.lib().idb_dedupe_noalloc(p, p, None, 0, None, 0, MAX_ROWS + 1, p, p, None)
    assert st == 4   # IDB_ERR_UNSUPPORTED, before touching any pointer
    assert "IDB_DEDUPE_NOALLOC_MAX_ROWS" in _lib.last_error()
