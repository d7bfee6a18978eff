"""Host-side mirror of the reference's InterlinkClass over the C ABI.

The reference's only host<->CUDA boundary is the InterlinkClass constructor
(cuda/Interlink.hpp:54-57, cuda/Interlink.cu:34-95): it takes the V calls, J
calls and sequences of the table, the two reference gene lists, the threshold,
minPts, the Hamming switch and the tree-statistics switch, clusters, and exposes
clusters / cores / uniques / copies through getters (cuda/Interlink.hpp:59-67).
``Interlink`` keeps those names and argument meanings; the work is done by
libimmunodbscan_gb300 (idb_cluster).  Errors surface as IdbError with the
library's status and message.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from typing import Optional, Sequence, Union

import numpy as np

from . import _lib
from ._lib import Input, Output, Params, Stats, check, lib

Strings = Union[Sequence[bytes], Sequence[str], tuple]


def _as_blob(strings) -> tuple:
    """(blob uint8, offsets int64) from a list of bytes/str or a (blob, offsets) pair."""
    if isinstance(strings, tuple) and len(strings) == 2 and isinstance(strings[0], np.ndarray):
        blob, off = strings
        return np.ascontiguousarray(blob, np.uint8), np.ascontiguousarray(off, np.int64)
    items = [s.encode() if isinstance(s, str) else bytes(s) for s in strings]
    off = np.zeros(len(items) + 1, np.int64)
    np.cumsum([len(s) for s in items], out=off[1:])
    blob = np.frombuffer(b"".join(items), dtype=np.uint8).copy()
    if blob.size == 0:
        blob = np.zeros(1, np.uint8)
    return blob, off


def _p(a) -> Optional[int]:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())   # torch tensor (device or pinned host)


class Context:
    """An idb_context: one device, one stream, a reusable workspace."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().idb_context_create(device, C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            lib().idb_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def make_params(threshold=float("nan"), abs_eps=-1, min_pts=2, use_hamming=False,
                eval_trees=False, schedule=0, tune=None, candidates=0,
                edge_memory_mb=0, row_chunks=0) -> Params:
    p = Params()
    p.threshold = float(threshold) if threshold is not None else math.nan
    p.abs_eps = int(abs_eps)
    p.min_pts = int(min_pts)
    p.use_hamming = int(bool(use_hamming))
    p.eval_trees = int(bool(eval_trees))
    p.schedule = int(schedule)
    if tune:
        p.tile_rx = int(tune[0])
        p.tile_ty = int(tune[1])
    p.candidates = int(candidates)
    p.edge_memory_mb = int(edge_memory_mb)
    p.row_chunks = int(row_chunks)
    return p


@dataclasses.dataclass
class Result:
    clone_id: np.ndarray
    core: np.ndarray
    copies: np.ndarray
    uniques: np.ndarray
    n_uniques: int
    tree_depth_hist: Optional[np.ndarray]
    stats: Stats


class Interlink:
    """Clusters one table; mirrors InterlinkClass(InputStrings, n_entries, V_genes_reference,
    V_gene_variant_count, J_genes_reference, J_gene_variant_count, threshold, minPts,
    use_only_hamming, eval_trees).

    ``v_calls`` / ``j_calls`` may be None (gene column not configured: every row
    matches the single gene "V", cpp/TableHolder.hpp:293-296); ``seqs`` may be
    None (every row is "Gene", cpp/TableHolder.hpp:326-328).  ``abs_eps`` is the
    added absolute threshold (-1 = unused); ``threshold`` may be NaN when only
    ``abs_eps`` is used.  ``rep_sizes`` splits the rows into independent
    repertoires (clone ids numbered per repertoire).
    """

    def __init__(self, v_calls, j_calls, seqs, n_entries: int, v_genes_reference,
                 j_genes_reference, threshold: float, min_pts: int, use_only_hamming: bool,
                 eval_trees: bool = False, *, abs_eps: int = -1, rep_sizes=None,
                 context: Optional[Context] = None, schedule: int = 0, tune=None,
                 candidates: int = 0, edge_memory_mb: int = 0, row_chunks: int = 0):
        n = int(n_entries)
        keep = []
        inp = Input()
        inp.n_rows = n

        def col(strings):
            if strings is None:
                return None, None
            blob, off = _as_blob(strings)
            if len(off) != n + 1:
                raise ValueError("column length differs from n_entries")
            keep.extend([blob, off])
            return _p(blob), _p(off)

        inp.v_calls, inp.v_offsets = col(v_calls)
        inp.j_calls, inp.j_offsets = col(j_calls)
        inp.seqs, inp.seq_offsets = col(seqs)

        def genes(names, present):
            if not present:
                return None, None, 0
            names = list(names)
            blob, off = _as_blob(names)
            keep.extend([blob, off])
            return _p(blob), _p(off), len(names)

        inp.v_genes, inp.v_gene_offsets, inp.n_v_genes = genes(v_genes_reference, v_calls is not None)
        inp.j_genes, inp.j_gene_offsets, inp.n_j_genes = genes(j_genes_reference, j_calls is not None)
        if rep_sizes is not None:
            roff = np.concatenate([[0], np.cumsum(rep_sizes)]).astype(np.uint32)
            keep.append(roff)
            inp.n_repertoires = len(rep_sizes)
            inp.rep_offsets = _p(roff)
        prm = make_params(threshold, abs_eps, min_pts, use_only_hamming, eval_trees, schedule, tune,
                          candidates, edge_memory_mb, row_chunks)
        self._result = _run(inp, prm, n, context, eval_trees)

    # getters of cuda/Interlink.hpp:59-63
    def get_clusters(self) -> np.ndarray:
        return self._result.clone_id

    def get_cores(self) -> np.ndarray:
        return self._result.core

    def get_uniques(self) -> np.ndarray:
        return self._result.uniques[: self._result.n_uniques]

    def get_copies(self) -> np.ndarray:
        return self._result.copies

    def get_n_uniques(self) -> int:
        return self._result.n_uniques

    @property
    def result(self) -> Result:
        return self._result


def _run(inp: Input, prm: Params, n: int, context: Optional[Context], trees: bool) -> Result:
    clone = np.zeros(max(n, 1), np.uint32)
    core = np.zeros(max(n, 1), np.int32)
    copies = np.zeros(max(n, 1), np.uint32)
    uniques = np.zeros(max(n, 1), np.uint32)
    nu = np.zeros(1, np.uint32)
    hist = np.zeros(51, np.uint32) if trees else None
    st = Stats()
    out = Output(_p(clone), _p(core), _p(copies), _p(uniques), _p(nu), _p(hist),
                 C.cast(C.pointer(st), C.c_void_p))
    h = context.handle if context is not None else None
    check(lib().idb_cluster(h, C.byref(inp), C.byref(prm), C.byref(out)))
    return Result(clone[:n], core[:n], copies[:n], uniques, int(nu[0]), hist, st)


def cluster_workload(w, context: Optional[Context] = None, *, schedule: int = 0, tune=None,
                     eval_trees: bool = False, no_v=False, no_j=False, no_seq=False) -> Result:
    """Cluster a synth.Workload (all its repertoires) through idb_cluster (host buffers)."""
    it = Interlink(None if no_v else (w.v_blob, w.v_off), None if no_j else (w.j_blob, w.j_off),
                   None if no_seq else (w.seq_blob, w.seq_off), w.n, w.v_genes, w.j_genes,
                   w.threshold, w.min_pts, w.use_hamming, eval_trees, abs_eps=w.abs_eps,
                   rep_sizes=np.diff(w.rep_off).tolist() if w.n_rep > 1 else None,
                   context=context, schedule=schedule, tune=tune,
                   candidates=w.candidates, edge_memory_mb=w.edge_memory_mb,
                   row_chunks=w.row_chunks)
    return it.result


class DeviceBatch:
    """Device-resident columns of a workload plus a captured batch plan.

    ``plan()`` runs idb_batch_plan (discovery run + CUDA graph capture of the whole
    path); ``run()`` replays the graph (idb_batch_run) and recomputes every output
    from the device inputs.  Requires torch for device memory.
    """

    def __init__(self, w, context: Context, *, schedule: int = 0, tune=None):
        import torch
        self.torch = torch
        self.ctx = context
        dev = torch.device("cuda", 0)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        self.seq, self.seq_off = t(w.seq_blob if w.seq_blob.size else np.zeros(1, np.uint8)), t(w.seq_off)
        self.v, self.v_off = t(w.v_blob), t(w.v_off)
        self.j, self.j_off = t(w.j_blob), t(w.j_off)
        n = w.n
        self.n = n
        self.clone = torch.zeros(n, dtype=torch.int32, device=dev)
        self.core = torch.zeros(n, dtype=torch.int32, device=dev)
        self.copies = torch.zeros(n, dtype=torch.int32, device=dev)
        self._keep = []
        inp = Input()
        inp.n_rows = n
        inp.seqs, inp.seq_offsets = _p(self.seq), _p(self.seq_off)
        inp.v_calls, inp.v_offsets = _p(self.v), _p(self.v_off)
        inp.j_calls, inp.j_offsets = _p(self.j), _p(self.j_off)
        vb, vo = _as_blob(w.v_genes)
        jb, jo = _as_blob(w.j_genes)
        roff = np.ascontiguousarray(w.rep_off, np.uint32)
        self._keep += [vb, vo, jb, jo, roff]
        inp.v_genes, inp.v_gene_offsets, inp.n_v_genes = _p(vb), _p(vo), len(w.v_genes)
        inp.j_genes, inp.j_gene_offsets, inp.n_j_genes = _p(jb), _p(jo), len(w.j_genes)
        inp.n_repertoires = w.n_rep
        inp.rep_offsets = _p(roff)
        self.inp = inp
        self.prm = make_params(w.threshold, w.abs_eps, w.min_pts, w.use_hamming, False, schedule, tune,
                               w.candidates, w.edge_memory_mb)
        self.out = Output(_p(self.clone), _p(self.core), _p(self.copies), None, None, None, None)

    def cluster_once(self) -> Stats:
        """idb_cluster_device: eager path on the device columns."""
        self.torch.cuda.synchronize()
        st = Stats()
        out = Output(self.out.clone_id, self.out.core, self.out.copies, None, None, None,
                     C.cast(C.pointer(st), C.c_void_p))
        check(lib().idb_cluster_device(self.ctx.handle, C.byref(self.inp), C.byref(self.prm),
                                       C.byref(out)))
        return st

    def plan(self) -> None:
        self.torch.cuda.synchronize()
        check(lib().idb_batch_plan(self.ctx.handle, C.byref(self.inp), C.byref(self.prm),
                                   C.byref(self.out)))

    def run(self) -> Stats:
        st = Stats()
        check(lib().idb_batch_run(self.ctx.handle, C.byref(st)))
        return st

    def results(self):
        return (self.clone.cpu().numpy().view(np.uint32), self.core.cpu().numpy(),
                self.copies.cpu().numpy().view(np.uint32))
