"""Runs the reference's own clustering path (oracle/_ref/ref_dbscan, built by
oracle/build_ref.py on the host execution model of oracle/ref_emu.h) on a
workload -- test infrastructure: it pins the oracle and feeds the golden
fixtures under tests/golden/.

The reference clusters one table per call, so a workload of several
repertoires runs one call per repertoire (clone ids are numbered per
repertoire, as the library numbers them).  The reference has no absolute eps:
only workloads with ``abs_eps < 0`` and a relative ``threshold`` can run.
"""
from __future__ import annotations

import dataclasses
import os
import struct
import subprocess
import sys
import tempfile
from typing import List, Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
if _HERE not in sys.path:
    sys.path.insert(0, _HERE)
import build_ref  # noqa: E402


@dataclasses.dataclass
class RefResult:
    clone_id: np.ndarray     # uint32 [n]
    core: np.ndarray         # int32 [n]
    copies: np.ndarray       # uint32 [n]
    uniques: np.ndarray      # uint32, ascending representative rows
    tree_depth_hist: Optional[List[np.ndarray]]   # one histogram per repertoire


def available() -> bool:
    return bool(build_ref.build())


def _encode(vcalls, jcalls, seqs, vg, jg, threshold, min_pts, use_hamming, eval_trees) -> bytes:
    parts = [b"IDBR", struct.pack("<I", len(seqs))]
    for col in (vcalls, jcalls, seqs):
        for s in col:
            parts.append(struct.pack("<I", len(s)))
            parts.append(s)
    for names in (vg, jg):
        parts.append(struct.pack("<I", len(names)))
        for s in names:
            parts.append(struct.pack("<I", len(s)))
            parts.append(s)
    parts.append(struct.pack("<fIII", threshold, min_pts, int(use_hamming), int(eval_trees)))
    return b"".join(parts)


def run_rows(vcalls, jcalls, seqs, vg, jg, threshold: float, min_pts: int, use_hamming: bool,
             eval_trees: bool = False):
    """One InterlinkClass call on lists of byte strings; returns
    (clone_id, core, copies, uniques, hist)."""
    exe = build_ref.build()
    if not exe:
        raise RuntimeError("IDB_REFERENCE_TREE does not name a reference tree")
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fin, "wb") as f:
            f.write(_encode(vcalls, jcalls, seqs, vg, jg, threshold, min_pts, use_hamming,
                            eval_trees))
        subprocess.run([exe, fin, fout], check=True, stdout=subprocess.DEVNULL)
        raw = np.fromfile(fout, dtype="<u4")
    n, nu = int(raw[0]), int(raw[1])
    p = 2
    clone = raw[p:p + n].astype(np.uint32); p += n
    core = raw[p:p + n].astype(np.int32); p += n
    copies = raw[p:p + n].astype(np.uint32); p += n
    uniq = raw[p:p + nu].astype(np.uint32); p += nu
    nh = int(raw[p]); p += 1
    hist = raw[p:p + nh].astype(np.uint32) if nh else None
    return clone, core, copies, uniq, hist


def run(w, eval_trees: bool = False) -> RefResult:
    """The reference's answer for a synth.Workload (relative threshold only)."""
    if w.abs_eps >= 0 or not np.isfinite(w.threshold):
        raise ValueError("the reference only has the relative threshold")
    clone, core, copies, uniq, hists = [], [], [], [], []
    for r in range(w.n_rep):
        lo, hi = int(w.rep_off[r]), int(w.rep_off[r + 1])
        rows = range(lo, hi)
        c, k, cp, u, h = run_rows([w.vcall(i) for i in rows], [w.jcall(i) for i in rows],
                                  [w.seq(i) for i in rows], w.v_genes, w.j_genes,
                                  float(w.threshold), int(w.min_pts), bool(w.use_hamming),
                                  eval_trees)
        clone.append(c); core.append(k); copies.append(cp); uniq.append(u + lo); hists.append(h)
    cat = lambda xs, t: np.concatenate(xs).astype(t) if xs else np.zeros(0, t)  # noqa: E731
    return RefResult(cat(clone, np.uint32), cat(core, np.int32), cat(copies, np.uint32),
                     cat(uniq, np.uint32), hists if eval_trees else None)
