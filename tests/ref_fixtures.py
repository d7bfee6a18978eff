"""The reference's own answers on small seeded cases (tests/golden/
ref_dbscan_cases.json.gz, written by tests/golden/make_ref_golden.py from the
reference's InterlinkClass run on the host execution model of oracle/ref_emu.h).

The reference's cluster growth lets the first core neighbour to win an
atomicCAS claim a border row (cuda/PSDBSCAN.hcu:113-122, :915-926).  The
fixtures come from one serial run, in which the core rows claim in ascending
order, so a border row carries its minimum-index core neighbour's cluster -- the
rule this library and the oracle use; the comparison is therefore exact.

The tree-depth histogram (cuda/PSDBSCAN.hcu:1020-1040) describes the
union-find forest, which depends on the union order in the reference too; the
parts that do not are its total (every row) and bin 0 (rows that are their own
root: noise uniques and one root per cluster).
"""
import gzip
import json
import os

import numpy as np

from immunodbscan_gb300 import synth

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_dbscan_cases.json.gz")


def load():
    with gzip.open(PATH, "rt") as f:
        data = json.load(f)
    out = []
    for c in data["cases"]:
        enc = lambda xs: [x.encode("latin-1") for x in xs]  # noqa: E731
        w = synth.from_strings(enc(c["seqs"]), enc(c["vcalls"]), enc(c["jcalls"]),
                               enc(c["v_genes"]), enc(c["j_genes"]), threshold=c["threshold"],
                               min_pts=c["min_pts"], use_hamming=c["use_hamming"],
                               rep_sizes=c["rep_sizes"])
        w.name = c["name"]
        want = {k: np.asarray(c[k], dtype=t) for k, t in
                (("clone_id", np.uint32), ("core", np.int32), ("copies", np.uint32),
                 ("uniques", np.uint32))}
        want["tree_depth_hist"] = [np.asarray(h, np.uint64) for h in c["tree_depth_hist"]]
        out.append((c["name"], w, want))
    return out


def names():
    return [n for n, _, _ in load()]


def assert_matches(name, want, clone_id, core, copies, uniques=None, hist=None):
    for key, got in (("copies", copies), ("core", core), ("clone_id", clone_id)):
        bad = np.nonzero(np.asarray(got) != want[key])[0]
        assert bad.size == 0, (f"{name}: {key} differs from the reference at {bad.size} rows, "
                               f"first {bad[:8].tolist()}: got {np.asarray(got)[bad[:8]].tolist()} "
                               f"want {want[key][bad[:8]].tolist()}")
    if uniques is not None:
        assert np.array_equal(np.asarray(uniques, np.uint32), want["uniques"]), f"{name}: uniques"
    if hist is not None:
        ref_total = sum(int(h.sum()) for h in want["tree_depth_hist"])
        ref_roots = sum(int(h[0]) for h in want["tree_depth_hist"])
        assert int(np.asarray(hist).sum()) == ref_total, f"{name}: histogram total"
        assert int(np.asarray(hist)[0]) == ref_roots, f"{name}: rows that are their own root"
