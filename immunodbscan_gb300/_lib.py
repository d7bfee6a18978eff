"""ctypes binding of the C ABI in include/immunodbscan_gb300.h.

The shared library is built in-tree (immunodbscan_gb300/_build/).  Loading
fails loudly when it is missing: there is no CPU fallback for the clustering.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libimmunodbscan_gb300.so")

IDB_OK = 0
MLP_FEATURES = 16
MLP_PARAMS = 16 * 64 + 64 + 64 * 64 + 64 + 64 + 1
STATUS_NAMES = {
    0: "IDB_OK", 1: "IDB_ERR_INVALID_ARG", 2: "IDB_ERR_CUDA", 3: "IDB_ERR_NO_DEVICE",
    4: "IDB_ERR_UNSUPPORTED", 5: "IDB_ERR_OUT_OF_MEMORY", 6: "IDB_ERR_CAPACITY",
    7: "IDB_ERR_DEVICE_STALL", 8: "IDB_ERR_REPLAN",
}


class IdbError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Params(C.Structure):
    _fields_ = [("threshold", C.c_float), ("abs_eps", C.c_int32), ("min_pts", C.c_uint32),
                ("use_hamming", C.c_int32), ("eval_trees", C.c_int32), ("schedule", C.c_int32),
                ("tile_rx", C.c_int32), ("tile_ty", C.c_int32), ("candidates", C.c_int32),
                ("edge_memory_mb", C.c_int32), ("row_chunks", C.c_int32),
                ("reserved", C.c_int32 * 1)]


class Tuning(C.Structure):
    _fields_ = [("tile_rx", C.c_int32), ("tile_ty", C.c_int32), ("ms_distance", C.c_double),
                ("n_tried", C.c_int32), ("tried_rx", C.c_int32 * 16), ("tried_ty", C.c_int32 * 16),
                ("tried_ms", C.c_double * 16), ("schedule", C.c_int32),
                ("schedule_ms", C.c_double * 2)]


class Input(C.Structure):
    _fields_ = [("n_rows", C.c_uint32),
                ("v_calls", C.c_void_p), ("v_offsets", C.c_void_p),
                ("j_calls", C.c_void_p), ("j_offsets", C.c_void_p),
                ("seqs", C.c_void_p), ("seq_offsets", C.c_void_p),
                ("v_genes", C.c_void_p), ("v_gene_offsets", C.c_void_p), ("n_v_genes", C.c_uint32),
                ("j_genes", C.c_void_p), ("j_gene_offsets", C.c_void_p), ("n_j_genes", C.c_uint32),
                ("n_repertoires", C.c_uint32), ("rep_offsets", C.c_void_p)]


class Stats(C.Structure):
    _fields_ = [("n_uniques", C.c_uint32), ("n_cores", C.c_uint32), ("n_clusters", C.c_uint32),
                ("n_noise_rows", C.c_uint32), ("pairs_evaluated", C.c_uint64),
                ("neighbour_pairs", C.c_uint64), ("n_entries", C.c_uint64), ("n_units", C.c_uint64),
                ("ms_total", C.c_double), ("ms_distance", C.c_double), ("ms_phase", C.c_double * 8),
                ("kernel_launches", C.c_uint32), ("core_edges", C.c_uint32),
                ("lev_columns", C.c_uint64), ("candidates", C.c_uint32), ("streamed", C.c_uint32)]


class Output(C.Structure):
    _fields_ = [("clone_id", C.c_void_p), ("core", C.c_void_p), ("copies", C.c_void_p),
                ("uniques", C.c_void_p), ("n_uniques", C.c_void_p),
                ("tree_depth_hist", C.c_void_p), ("stats", C.c_void_p)]


# exported functions and their signatures (kept in step with the header)
SIGNATURES = {
    "idb_context_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "idb_context_destroy": (C.c_int, [C.c_void_p]),
    "idb_cluster": (C.c_int, [C.c_void_p, C.POINTER(Input), C.POINTER(Params), C.POINTER(Output)]),
    "idb_cluster_device": (C.c_int, [C.c_void_p, C.POINTER(Input), C.POINTER(Params),
                                     C.POINTER(Output)]),
    "idb_batch_plan": (C.c_int, [C.c_void_p, C.POINTER(Input), C.POINTER(Params),
                                 C.POINTER(Output)]),
    "idb_batch_run": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "idb_last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "idb_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "idb_host_free": (C.c_int, [C.c_void_p]),
    "idb_diag_eps": (C.c_int32, [C.c_uint32, C.c_uint32, C.c_float, C.c_int32]),
    "idb_diag_eps_hops": (C.c_int32, [C.c_uint32, C.c_uint32, C.c_float, C.c_int32, C.c_int32]),
    "idb_status_string": (C.c_char_p, [C.c_int]),
    "idb_abi_version": (C.c_int, []),
    "idb_dedupe_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                     C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "idb_autotune": (C.c_int, [C.c_void_p, C.POINTER(Input), C.POINTER(Params), C.POINTER(Tuning)]),
    "idb_profile_binpairs": (C.c_int, [C.c_void_p, C.POINTER(Input), C.POINTER(Params), C.c_void_p,
                                       C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "idb_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_float,
                                C.c_void_p, C.POINTER(C.c_float)]),
    "idb_mlp_load": (C.c_int, [C.c_void_p, C.c_void_p]),
    "idb_diag_mlp_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                    C.c_void_p, C.POINTER(C.c_float)]),
    "idb_diag_mlp_predict": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                       C.c_void_p]),
    "idb_diag_int_peak": (C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "idb_diag_gene_bits": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                     C.c_void_p, C.c_uint32, C.c_void_p]),
    "idb_count_admissible": (C.c_int, [C.c_void_p, C.POINTER(Input), C.POINTER(Params),
                                       C.POINTER(C.c_uint64)]),
}

_lib = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m immunodbscan_gb300.build` "
                "(the clustering path has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().idb_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    if status != IDB_OK:
        raise IdbError(status, last_error())
