"""The CPU oracle against the hand-derived known answers (rules S1-S7).

These pin the oracle (the reference ships no tests or fixtures; its CUDA path
cannot run here), which then serves as the checker for the GPU path.
"""
import os
import sys

import numpy as np
import pytest

import oracle
from kat_cases import S1_CALLS, S1_GENES, S1_WORDS, S2_TABLE, cases, no_seq_case


def test_s1_gene_bitsets():
    got = oracle.gene_bitsets(S1_CALLS, S1_GENES)
    assert got.tolist() == S1_WORDS


def test_s1_width_is_ceil_genes_over_32():
    genes = [b"G%d*" % g for g in range(40)]
    got = oracle.gene_bitsets([b"xG39*", b"G0*G1*"], genes)
    assert got.shape == (2, 2)
    assert got[0].tolist() == [0, 1 << 7]
    assert got[1].tolist() == [3, 0]


@pytest.mark.parametrize("lx,ly,t,a,want", S2_TABLE)
def test_s2_eps(lx, ly, t, a, want):
    assert oracle.eps(lx, ly, t, a) == want


def test_s4_distances():
    assert oracle.levenshtein(b"kitten", b"sitting") == 3
    assert oracle.levenshtein(b"ACDEFGHIKL", b"ACDFGHIKLM") == 2
    assert oracle.levenshtein(b"ACDEFGHIK", b"ACDFGHIKLM") == 3
    assert oracle.levenshtein(b"ACDFGHIKLM", b"ACDEFGHIKLMN") == 2
    assert oracle.levenshtein(b"", b"ABC") == 3
    assert oracle.hamming(b"ACDFGHIKLM", b"ACDEFGHIKL") == 7


@pytest.mark.parametrize("case", cases(), ids=lambda c: c["name"])
def test_known_answers(case):
    r = oracle.cluster(case["w"])
    assert r.clone_id.tolist() == case["clone"]
    assert r.core.tolist() == case["core"]
    assert r.copies.tolist() == case["copies"]
    for row, labels in case["cand"].items():
        assert r.n_cand[row] == len(labels)
        assert sorted(r.cand[row, : len(labels)].tolist()) == labels


def test_no_sequence_column():
    w, want = no_seq_case()
    r = oracle.cluster(w, no_seq=True)
    assert r.clone_id.tolist() == want["clone"]
    assert r.core.tolist() == want["core"]
    assert r.copies.tolist() == want["copies"]


def test_no_gene_columns_equals_single_gene_v():
    from immunodbscan_gb300 import synth
    w = synth.workload(0, scale=0.05)
    a = oracle.cluster(w, no_v=True, no_j=True)
    w2 = synth.from_strings([w.seq(i) for i in range(w.n)], None, None, [], [],
                            abs_eps=w.abs_eps, min_pts=w.min_pts, use_hamming=w.use_hamming)
    b = oracle.cluster(w2)
    assert np.array_equal(a.clone_id, b.clone_id)
    assert np.array_equal(a.copies, b.copies)


def test_invariants_workload0():
    """Properties that hold for any input: copies sum to the row count, duplicates
    carry copies 0 and follow their representative, labels are dense 1..K."""
    from immunodbscan_gb300 import synth
    w = synth.workload(0, scale=0.2)
    r = oracle.cluster(w)
    assert int(r.copies.sum()) == w.n
    assert (r.copies > 0).sum() == r.n_uniques
    labs = np.unique(r.clone_id[r.clone_id > 0])
    assert labs.tolist() == list(range(1, r.n_clusters + 1))
    # core rows are representatives (minPts > 0) and are never noise
    assert np.all(r.copies[r.core == 1] > 0)
    assert np.all(r.clone_id[r.core == 1] > 0)
    # labels ascend with the first core row of each cluster
    first = {}
    for i in np.nonzero(r.core)[0]:
        first.setdefault(int(r.clone_id[i]), int(i))
    order = [first[k] for k in sorted(first)]
    assert order == sorted(order)


def _eps_golden():
    import gzip
    import json
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "eps_reference.json.gz")
    with gzip.open(path, "rt") as f:
        return json.load(f)


def test_eps_matches_reference_functor():
    """The oracle's threshold rule against the reference's own
    epsilonOneFunctorClass, compiled from its header (golden table made by
    tests/golden/make_eps_golden.py): every length pair up to 64 for the
    Levenshtein functor and equal lengths up to 1024 for the Hamming one."""
    g = _eps_golden()
    n = g["max_len"]
    for k, t in enumerate(g["thresholds"]):
        lev = g["levenshtein"][k]
        for q in range(n + 1):
            for s in range(n + 1):
                assert oracle.eps(q, s, t) == lev[q][s], (t, q, s)
        ham = g["hamming"][k]
        for q in range(0, g["diag_len"] + 1, 7):
            assert oracle.eps(q, q, t) == ham[q], (t, q)


def test_library_eps_matches_reference_functor():
    """The threshold the library tabulates for its kernels (host code, no device
    needed) against the same reference table."""
    import ctypes as C
    from immunodbscan_gb300 import _lib
    L = _lib.lib()
    g = _eps_golden()
    n = g["max_len"]
    for k, t in enumerate(g["thresholds"]):
        lev = g["levenshtein"][k]
        for q in range(n + 1):
            for s in range(n + 1):
                assert L.idb_diag_eps(q, s, C.c_float(t), -1) == lev[q][s], (t, q, s)
        ham = g["hamming"][k]
        for q in range(g["diag_len"] + 1):
            assert L.idb_diag_eps(q, q, C.c_float(t), -1) == ham[q], (t, q)


def test_library_multi_hop_bounds_match_reference_functors():
    """The two- and three-hop bounds (idb_diag_eps_hops) against the reference's
    epsilonTwoFunctorClass / epsilonThreeFunctorClass, entry by entry, in both
    the Levenshtein and the equal-length Hamming form."""
    import ctypes as C
    from immunodbscan_gb300 import _lib
    L = _lib.lib()
    g = _eps_golden()
    n = g["max_len"]
    for k, t in enumerate(g["thresholds"]):
        ft = C.c_float(t)
        for hops, key in ((2, "two_hop"), (3, "three_hop")):
            tab = g[key][k]
            for q in range(n + 1):
                for s in range(n + 1):
                    assert L.idb_diag_eps_hops(q, s, ft, hops, 0) == tab[q][s], (key, t, q, s)
        h2, h3 = g["hamming_two_three"][k]
        for q in range(len(h2)):
            assert L.idb_diag_eps_hops(q, q, ft, 2, 1) == h2[q], ("hamming two", t, q)
            assert L.idb_diag_eps_hops(q, q, ft, 3, 1) == h3[q], ("hamming three", t, q)


@pytest.mark.parametrize("t", [0.1, 0.15, 0.25])
def test_multi_hop_bound_holds_on_neighbour_chains(t):
    """What the bounds promise: sequences joined through one (two) intermediate
    neighbours under the relative threshold are within the two-hop (three-hop)
    bound of each other, by the oracle's edit distance."""
    import ctypes as C
    from immunodbscan_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(int(t * 1000))
    alpha = list(b"ACDEFGHIKLMNPQRSTVWY")

    def mutate(x, k):
        x = bytearray(x)
        for _ in range(k):
            op = rng.integers(0, 3)
            if op == 0 and x:
                x[int(rng.integers(0, len(x)))] = int(rng.choice(alpha))
            elif op == 1 and len(x) > 1:
                del x[int(rng.integers(0, len(x)))]
            else:
                x.insert(int(rng.integers(0, len(x) + 1)), int(rng.choice(alpha)))
        return bytes(x)

    def near(a, b):
        return oracle.levenshtein(a, b) <= oracle.eps(len(a), len(b), t, -1)

    chains = 0
    for _ in range(3000):
        x = bytes(rng.choice(alpha, size=int(rng.integers(8, 30))).astype(np.uint8))
        b = mutate(x, int(rng.integers(0, 5)))
        c = mutate(b, int(rng.integers(0, 5)))
        y = mutate(c, int(rng.integers(0, 5)))
        if near(x, b) and near(b, c):
            chains += 1
            assert oracle.levenshtein(x, c) <= L.idb_diag_eps_hops(len(x), len(c), C.c_float(t), 2, 0)
            if near(c, y):
                assert oracle.levenshtein(x, y) <= L.idb_diag_eps_hops(len(x), len(y), C.c_float(t), 3, 0)
    assert chains > 100


def _segments(L, S):
    return [(k * L // S, (k + 1) * L // S) for k in range(S)]


@pytest.mark.parametrize("eps", [0, 1, 2])
def test_segment_join_rule_emits_each_neighbour_pair_once(eps):
    """The segment join's rule (k_buckets.cu join kernels, k_distance.cu
    emission), restated on the host: with S = eps+1 segments
    [kL/S, (k+1)L/S), two equal-length sequences within Hamming eps share at
    least one identical segment, and exactly one group k passes the emission
    test (segment k identical, no lower segment identical).  Includes lengths
    below S (empty segments) and identical sequences."""
    rng = np.random.default_rng(eps)
    S = eps + 1
    checked = 0
    for _ in range(4000):
        L = int(rng.integers(1, 40))
        x = rng.integers(0, 4, size=L)
        y = x.copy()
        for p in rng.choice(L, size=min(L, int(rng.integers(0, eps + 1))), replace=False):
            y[p] = (y[p] + 1 + rng.integers(0, 3)) % 4
        assert int(np.sum(x != y)) <= eps
        same = [bool(np.array_equal(x[lo:hi], y[lo:hi])) for lo, hi in _segments(L, S)]
        assert any(same)                                    # pigeonhole
        emit = [same[k] and not any(same[:k]) for k in range(S)]
        assert sum(emit) == 1                               # emitted exactly once
        checked += 1
    assert checked == 4000


# --- the oracle against the reference's own code -------------------------------

import ref_fixtures  # noqa: E402


@pytest.mark.parametrize("name", ref_fixtures.names())
def test_oracle_matches_reference_fixtures(name):
    """Golden answers of the reference's InterlinkClass (relative threshold,
    Hamming and Levenshtein modes, minPts 0-5, ambiguous and unmatched gene
    calls, missing gene columns, several repertoires)."""
    _, w, want = next(c for c in ref_fixtures.load() if c[0] == name)
    r = oracle.cluster(w)
    ref_fixtures.assert_matches(name, want, r.clone_id, r.core, r.copies,
                                uniques=np.nonzero(r.copies)[0])


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_oracle_matches_live_reference(seed):
    """Fresh random cases through the reference's own code, when its tree is
    available (IDB_REFERENCE_TREE); the fixtures above cover every other run."""
    import ref_run
    if not ref_run.available():
        pytest.skip("IDB_REFERENCE_TREE does not name a reference tree")
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_ref_golden import _random_case
    rng = np.random.default_rng(seed)
    hamming = bool(seed % 2)
    alphabet = list(b"ACGT") if seed != 12 else list(b"ACDEFGHIKLMNPQRSTVWY")
    w = _random_case(seed, 300, 4, 10, alphabet, hamming, float(rng.choice([0.1, 0.2, 0.3])),
                     int(rng.integers(1, 5)), 30)
    want = ref_run.run(w)
    r = oracle.cluster(w)
    assert np.array_equal(r.copies, want.copies)
    assert np.array_equal(r.core, want.core)
    assert np.array_equal(r.clone_id, want.clone_id)


def test_levenshtein_cutoff_matches_full_dp():
    rng = np.random.default_rng(3)
    for _ in range(4000):
        a = bytes(rng.choice(list(b"ACGT"), size=int(rng.integers(0, 14))).astype(np.uint8))
        b = bytearray(a)
        for _ in range(int(rng.integers(0, 5))):
            op = rng.integers(0, 3)
            if op == 0 and b:
                b[int(rng.integers(0, len(b)))] = int(rng.choice(list(b"ACGT")))
            elif op == 1 and b:
                del b[int(rng.integers(0, len(b)))]
            else:
                b.insert(int(rng.integers(0, len(b) + 1)), int(rng.choice(list(b"ACGT"))))
        b = bytes(b)
        d = oracle.levenshtein(a, b)
        for e in range(-1, 6):
            assert oracle.levenshtein_within(a, b, e) == (d <= e), (a, b, e, d)


@pytest.mark.parametrize("k,scale,threshold", [(1, 0.01, None), (3, 0.005, None),
                                               (4, 0.001, None), (0, 0.3, 0.15), (2, 0.01, 0.1)])
def test_indexed_mode_matches_all_pairs(k, scale, threshold):
    """The oracle's indexed mode (length-windowed pairs, cutoff DP) gives the
    all-pairs answer, so it can check inputs too large for the full mode."""
    from immunodbscan_gb300 import synth
    w = synth.workload(k, scale=scale)
    if threshold is not None:
        w.abs_eps, w.threshold = -1, threshold
    a = oracle.cluster(w)
    b = oracle.cluster(w, indexed=True)
    assert np.array_equal(a.clone_id, b.clone_id)
    assert np.array_equal(a.core, b.core)
    assert np.array_equal(a.copies, b.copies)
    assert (a.admissible_pairs, a.neighbour_pairs) == (b.admissible_pairs, b.neighbour_pairs)
