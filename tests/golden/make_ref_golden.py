"""Writes tests/golden/ref_dbscan_cases.json.gz: inputs and the reference's own
answers (clone_id, cores, copies, uniques, tree-depth histogram) for a set of
small seeded cases, computed by the reference's clustering translation unit
(cuda/Interlink.cu and its headers) run on the host execution model of
oracle/ref_emu.h.  Run where the reference tree is present:

    IDB_REFERENCE_TREE=<reference checkout> python tests/golden/make_ref_golden.py

The reference has only the relative threshold (maximum_relative_edit_distance),
so every case uses it; the absolute eps of this library is checked against the
oracle elsewhere.
"""
import gzip
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import ref_run  # noqa: E402
from immunodbscan_gb300 import synth  # noqa: E402


def _random_case(seed, n, lo, hi, alphabet, hamming, threshold, min_pts, n_fam, genes=True):
    """Families of short strings over a small alphabet: many duplicates, dense
    neighbourhoods, ambiguous calls, calls matching no gene, border rows.

    With minPts 0 every row is a core row, duplicates included, and the
    reference's grow_clusters then writes more core indices than its buffer
    holds (core_point_indices has n_uniques entries, the copy_if at
    cuda/PSDBSCAN.hcu:1191-1194 writes one per core row): out of bounds.  Those
    cases are drawn without duplicate sequences."""
    rng = np.random.default_rng(seed)
    roots = [bytes(rng.choice(alphabet, size=int(rng.integers(lo, hi + 1))).astype(np.uint8))
             for _ in range(n_fam)]
    seqs = []
    for _ in range(n):
        s = bytearray(roots[int(rng.integers(0, n_fam))])
        for _ in range(int(rng.poisson(0.8))):
            s[int(rng.integers(0, len(s)))] = int(rng.choice(alphabet))
        if not hamming and rng.random() < 0.15 and len(s) > lo:
            del s[int(rng.integers(0, len(s)))]
        if not hamming and rng.random() < 0.1:
            s.insert(int(rng.integers(0, len(s) + 1)), int(rng.choice(alphabet)))
        seqs.append(bytes(s))
    if min_pts == 0:
        seqs = list(dict.fromkeys(seqs))
        n = len(seqs)
    if not genes:
        return synth.from_strings(seqs, None, None, [], [], threshold=threshold,
                                  min_pts=min_pts, use_hamming=hamming)
    vg = [b"IGHV%d-%d*" % (a, b) for a in range(1, 6) for b in range(1, 4)]       # 15
    jg = [b"IGHJ%d*" % a for a in range(1, 5)]
    vc, jc = [], []
    for _ in range(n):
        r = rng.random()
        if r < 0.05:
            vc.append(b"IGHV9-9*01")          # matches no gene: compatible with nobody
        else:
            k = 1 + int(rng.integers(0, 3))
            picks = rng.choice(len(vg), size=k, replace=False)
            vc.append(b", or ".join(b"Homsap " + vg[int(g)] + b"0%d F" % (1 + rng.integers(0, 3))
                                    for g in picks))
        jc.append(b"Homsap " + jg[int(rng.integers(0, len(jg)))] + b"01 F")
    return synth.from_strings(seqs, vc, jc, vg, jg, threshold=threshold, min_pts=min_pts,
                              use_hamming=hamming)


def _workload(k, scale, threshold, hamming, min_pts=None):
    w = synth.workload(k, scale=scale)
    w.abs_eps = -1
    w.threshold = threshold
    w.use_hamming = hamming
    if min_pts is not None:
        w.min_pts = min_pts
    return w


def cases():
    aa, nt = list(b"ACDEFGHIKLMNPQRSTVWY"), list(b"ACGT")
    return [
        ("w0_hamming_t0.10", _workload(0, 0.05, 0.10, True)),
        ("w0_levenshtein_t0.15", _workload(0, 0.05, 0.15, False)),
        ("w1_levenshtein_t0.05", _workload(1, 0.004, 0.05, False)),
        ("w1_hamming_t0.06", _workload(1, 0.004, 0.06, True)),
        ("w2_hamming_t0.10_reps", _workload(2, 0.0006, 0.10, True)),
        ("w3_levenshtein_t0.15", _workload(3, 0.0006, 0.15, False)),
        ("w4_levenshtein_t0.15_minpts4", _workload(4, 0.0001, 0.15, False)),
        ("rand_nt_hamming_t0.25_minpts2", _random_case(1, 600, 4, 9, nt, True, 0.25, 2, 40)),
        ("rand_nt_levenshtein_t0.25_minpts3", _random_case(2, 600, 4, 9, nt, False, 0.25, 3, 40)),
        ("rand_aa_levenshtein_t0.2_minpts1", _random_case(3, 500, 6, 12, aa, False, 0.2, 1, 60)),
        ("rand_aa_hamming_t0.2_minpts0", _random_case(4, 400, 6, 12, aa, True, 0.2, 0, 60)),
        ("rand_aa_levenshtein_t0.2_minpts0", _random_case(5, 400, 6, 12, aa, False, 0.2, 0, 60)),
        ("rand_nt_levenshtein_t0.3_minpts5", _random_case(6, 600, 3, 8, nt, False, 0.3, 5, 30)),
        ("rand_aa_hamming_t0.0_minpts2", _random_case(7, 500, 5, 9, aa, True, 0.0, 2, 50)),
        ("rand_nt_levenshtein_nogenes_t0.2", _random_case(8, 500, 4, 10, nt, False, 0.2, 3, 40,
                                                           genes=False)),
        ("rand_aa_hamming_nogenes_t0.2", _random_case(9, 500, 5, 10, aa, True, 0.2, 2, 40,
                                                      genes=False)),
    ]


def main():
    if not ref_run.available():
        sys.exit("IDB_REFERENCE_TREE does not name a reference tree")
    out = {"source": "cuda/Interlink.cu (InterlinkClass) of the reference, run by "
                     "oracle/_ref/ref_dbscan (oracle/build_ref.py, oracle/ref_emu.h)",
           "cases": []}
    for name, w in cases():
        t = time.time()
        r = ref_run.run(w, eval_trees=True)
        dec = lambda xs: [x.decode("latin-1") for x in xs]  # noqa: E731
        out["cases"].append({
            "name": name,
            "seqs": dec(w.seq(i) for i in range(w.n)),
            "vcalls": dec(w.vcall(i) for i in range(w.n)),
            "jcalls": dec(w.jcall(i) for i in range(w.n)),
            "v_genes": dec(w.v_genes), "j_genes": dec(w.j_genes),
            "rep_sizes": np.diff(w.rep_off).astype(int).tolist(),
            "threshold": float(w.threshold), "min_pts": int(w.min_pts),
            "use_hamming": bool(w.use_hamming),
            "clone_id": r.clone_id.tolist(), "core": r.core.tolist(),
            "copies": r.copies.tolist(), "uniques": r.uniques.tolist(),
            "tree_depth_hist": [h.tolist() for h in r.tree_depth_hist],
        })
        print("%-36s %6d rows %5d clusters %6.1f s" % (name, w.n, int(r.clone_id.max(initial=0)),
                                                       time.time() - t))
    path = os.path.join(HERE, "ref_dbscan_cases.json.gz")
    with gzip.open(path, "wt") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
