"""Autotuner front end: work-unit shapes picked per workload class, cached on disk.

``idb_autotune`` (C ABI) builds the buckets of a workload once and times the
distance kernel for every candidate shape (x-entries per lane, y-chunk length).
This module keys the result by the workload's class -- distance mode, threshold,
longest sequence in 32-residue words, alphabet size class and the order of
magnitude of the row count -- and keeps it in a JSON cache, so repeated runs on
similar data reuse the measured choice.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
from typing import Optional, Tuple

import numpy as np

from . import _lib
from .interlink import Context, make_params

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "immunodbscan_gb300", "tuning.json")


def workload_key(w) -> str:
    L = int(w.lengths().max()) if w.n else 0
    codes = len(np.unique(w.seq_blob[: 1 << 20])) if w.seq_blob.size else 1
    return json.dumps({
        "mode": "hamming" if w.use_hamming else "levenshtein",
        "eps": [None if math.isnan(w.threshold) else round(float(w.threshold), 4), int(w.abs_eps)],
        "words": max(1, (L + 31) // 32),
        "codes": "<=4" if codes <= 4 else ("<=32" if codes <= 32 else ">32"),
        "rows_log10": int(math.log10(max(w.n, 1))),
        "candidates": int(w.candidates),
    }, sort_keys=True)


def _input(w):
    from .interlink import _as_blob
    keep = []

    def arr(a):
        a = np.ascontiguousarray(a)
        keep.append(a)
        return a.ctypes.data

    inp = _lib.Input()
    inp.n_rows = w.n
    inp.seqs, inp.seq_offsets = arr(w.seq_blob if w.seq_blob.size else np.zeros(1, np.uint8)), arr(w.seq_off)
    inp.v_calls, inp.v_offsets = arr(w.v_blob), arr(w.v_off)
    inp.j_calls, inp.j_offsets = arr(w.j_blob), arr(w.j_off)
    vb, vo = _as_blob(w.v_genes)
    jb, jo = _as_blob(w.j_genes)
    inp.v_genes, inp.v_gene_offsets, inp.n_v_genes = arr(vb), arr(vo), len(w.v_genes)
    inp.j_genes, inp.j_gene_offsets, inp.n_j_genes = arr(jb), arr(jo), len(w.j_genes)
    inp.n_repertoires = w.n_rep
    inp.rep_offsets = arr(np.ascontiguousarray(w.rep_off, np.uint32))
    return inp, keep


def measure(w, ctx: Optional[Context] = None) -> dict:
    """Run idb_autotune on the workload; returns the best shape and all timings."""
    inp, keep = _input(w)
    prm = make_params(w.threshold, w.abs_eps, w.min_pts, w.use_hamming,
                      candidates=w.candidates)
    t = _lib.Tuning()
    _lib.check(_lib.lib().idb_autotune(ctx.handle if ctx else None, C.byref(inp), C.byref(prm),
                                       C.byref(t)))
    tried = [{"rx": t.tried_rx[k], "ty": t.tried_ty[k], "ms": t.tried_ms[k]} for k in range(t.n_tried)]
    return {"rx": t.tile_rx, "ty": t.tile_ty, "ms": t.ms_distance, "tried": tried,
            "schedule": t.schedule, "schedule_ms": [t.schedule_ms[0], t.schedule_ms[1]]}


def shape_for(w, ctx: Optional[Context] = None, cache_path: str = DEFAULT_CACHE,
              refresh: bool = False) -> Tuple[int, int, dict]:
    """(tile_rx, tile_ty, record) for the workload, measuring once per workload class."""
    key = workload_key(w)
    cache = {}
    if os.path.exists(cache_path):
        try:
            with open(cache_path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    if refresh or key not in cache:
        cache[key] = measure(w, ctx)
        os.makedirs(os.path.dirname(cache_path) or ".", exist_ok=True)
        tmp = cache_path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, cache_path)
    rec = cache[key]
    return int(rec["rx"]), int(rec["ty"]), rec
