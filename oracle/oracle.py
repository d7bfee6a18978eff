"""ctypes wrapper of the CPU oracle (test infrastructure; see oracle.h).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline / reference arm
use this module, as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
if _HERE not in sys.path:
    sys.path.insert(0, _HERE)
import build_oracle  # noqa: E402

_lib = None


class _Params(C.Structure):
    _fields_ = [("threshold", C.c_float), ("abs_eps", C.c_int32), ("min_pts", C.c_uint32),
                ("use_hamming", C.c_int32), ("n_threads", C.c_int32),
                ("max_candidates", C.c_int32), ("indexed", C.c_int32)]


class _Result(C.Structure):
    _fields_ = [("clone_id", C.c_void_p), ("core", C.c_void_p), ("copies", C.c_void_p),
                ("cand", C.c_void_p), ("n_cand", C.c_void_p),
                ("n_uniques", C.c_uint32), ("n_cores", C.c_uint32), ("n_clusters", C.c_uint32),
                ("admissible_pairs", C.c_uint64), ("neighbour_pairs", C.c_uint64),
                ("all_pairs", C.c_uint64)]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        L.ora_cluster.restype = C.c_int
        L.ora_eps.restype = C.c_int32
        L.ora_eps.argtypes = [C.c_uint32, C.c_uint32, C.c_float, C.c_int32]
        L.ora_levenshtein.restype = C.c_int32
        L.ora_levenshtein.argtypes = [C.c_char_p, C.c_uint32, C.c_char_p, C.c_uint32]
        L.ora_hamming.restype = C.c_int32
        L.ora_hamming.argtypes = [C.c_char_p, C.c_char_p, C.c_uint32]
        L.ora_levenshtein_within.restype = C.c_int32
        L.ora_levenshtein_within.argtypes = [C.c_char_p, C.c_uint32, C.c_char_p, C.c_uint32,
                                             C.c_int32]
        L.ora_gene_bitsets.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _genes(names):
    blob = np.frombuffer(b"".join(names), dtype=np.uint8).copy() if names else np.zeros(1, np.uint8)
    off = np.zeros(len(names) + 1, np.int64)
    np.cumsum([len(g) for g in names], out=off[1:])
    return blob, off


@dataclasses.dataclass
class OracleResult:
    clone_id: np.ndarray
    core: np.ndarray
    copies: np.ndarray
    cand: np.ndarray          # [n, K]
    n_cand: np.ndarray
    n_uniques: int
    n_cores: int
    n_clusters: int
    admissible_pairs: int
    neighbour_pairs: int
    all_pairs: int


def cluster(w, *, n_threads: int = 0, max_candidates: int = 8, no_v=False, no_j=False,
            no_seq=False, indexed: bool = False) -> OracleResult:
    """Run the oracle on a synth.Workload (all repertoires).  ``indexed``
    pairs only uniques within the largest admissible length gap and stops the
    edit distance at eps: the same answer, for large inputs; the default keeps
    the reference's all-pairs, full-DP structure."""
    L = lib()
    n = w.n
    vgb, vgo = _genes(w.v_genes)
    jgb, jgo = _genes(w.j_genes)
    prm = _Params(float(w.threshold), int(w.abs_eps), int(w.min_pts), int(bool(w.use_hamming)),
                  int(n_threads), int(max_candidates), int(bool(indexed)))
    K = max(int(max_candidates), 0)
    clone = np.zeros(n, np.uint32)
    core = np.zeros(n, np.int32)
    copies = np.zeros(n, np.uint32)
    cand = np.zeros((n, max(K, 1)), np.uint32)
    ncand = np.zeros(n, np.uint32)
    res = _Result(_p(clone), _p(core), _p(copies), _p(cand), _p(ncand), 0, 0, 0, 0, 0, 0)
    seq_blob = w.seq_blob if w.seq_blob.size else np.zeros(1, np.uint8)
    v_blob = w.v_blob if w.v_blob.size else np.zeros(1, np.uint8)
    j_blob = w.j_blob if w.j_blob.size else np.zeros(1, np.uint8)
    rc = L.ora_cluster(
        C.c_uint32(n),
        None if no_v else _p(v_blob), None if no_v else _p(w.v_off),
        None if no_j else _p(j_blob), None if no_j else _p(w.j_off),
        None if no_seq else _p(seq_blob), None if no_seq else _p(w.seq_off),
        _p(vgb), _p(vgo), C.c_uint32(len(w.v_genes)),
        _p(jgb), _p(jgo), C.c_uint32(len(w.j_genes)),
        C.c_uint32(w.n_rep), _p(np.ascontiguousarray(w.rep_off, np.uint32)),
        C.byref(prm), C.byref(res))
    if rc != 0:
        raise RuntimeError(f"ora_cluster failed: {rc}")
    return OracleResult(clone, core, copies, cand[:, :K], ncand, res.n_uniques, res.n_cores,
                        res.n_clusters, res.admissible_pairs, res.neighbour_pairs, res.all_pairs)


def eps(lx: int, ly: int, threshold: float = float("nan"), abs_eps: int = -1) -> int:
    return int(lib().ora_eps(lx, ly, threshold, abs_eps))


def levenshtein(a: bytes, b: bytes) -> int:
    return int(lib().ora_levenshtein(a, len(a), b, len(b)))


def levenshtein_within(a: bytes, b: bytes, e: int) -> bool:
    return bool(lib().ora_levenshtein_within(a, len(a), b, len(b), e))


def hamming(a: bytes, b: bytes) -> int:
    assert len(a) == len(b)
    return int(lib().ora_hamming(a, b, len(a)))


def gene_bitsets(calls, genes) -> np.ndarray:
    """Reference-layout int32 bitset words, shape [n, ceil(G/32)]."""
    cb, co = _genes(list(calls))
    gb, go = _genes(list(genes))
    width = (len(genes) + 31) // 32
    out = np.zeros((len(calls), max(width, 1)), np.uint32)
    lib().ora_gene_bitsets(C.c_uint32(len(calls)), _p(cb), _p(co), _p(gb), _p(go),
                           C.c_uint32(len(genes)), _p(out))
    return out[:, :width]


NAN = math.nan
