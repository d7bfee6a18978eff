"""Known-answer cases for rules S1-S7, derived by hand from the reference.

The reference ships no tests and no example data, so these cases pin both the
CPU oracle and the GPU path.  Each case states the rule it exercises and the
reference lines the expected values follow; the expected arrays were worked out
by hand (pairwise distances are listed in the comments).
"""
import math

from immunodbscan_gb300.synth import from_strings

NAN = math.nan
V3 = [b"IGHV1-2*", b"IGHV1-24*", b"IGHV3-23*"]

# S1: bit g set iff gene name g is a byte-exact, case-sensitive substring of the
# call (cuda/BitsetVector.inl:149-175); names end in '*' so IGHV1-2* does not
# match IGHV1-24* (cpp/GeneReader.hpp:43-46).  Reference layout: int32 words.
S1_CALLS = [b"Homsap IGHV1-2*01 F", b"Homsap IGHV1-24*01 F", b"IGHV1-2*01, or IGHV3-23*02",
            b"ighv1-2*01", b"", b"IGHV1-2", b"IGHV3-23*01 F, or Homsap IGHV1-24*03 F"]
S1_GENES = V3
S1_WORDS = [[1], [2], [5], [0], [0], [0], [6]]

# S2: eps = (int)truncf((float)max(Lx,Ly) * t) in single precision
# (cuda/SpecialFunctors.hcu:257-261); abs caps it (added key).
# (lx, ly, threshold, abs_eps, expected)
S2_TABLE = [
    (16, 16, 0.15, -1, 2),     # 2.4
    (20, 20, 0.15, -1, 3),     # 20*0.15f = 3.0000002 -> 3
    (13, 7, 0.15, -1, 1),      # 1.95
    (6, 6, 0.15, -1, 0),       # 0.9
    (10, 9, 0.2, -1, 2),       # 2.0000000 in float
    (12, 10, 0.2, -1, 2),      # 2.4
    (100, 100, 0.29, -1, 29),  # 0.29f*100 rounds to 29.0 in float (28.99999916 in double)
    (30, 30, 0.15, 3, 3),      # min(3, 4)
    (16, 16, 0.15, 3, 2),      # min(3, 2)
    (25, 25, NAN, 1, 1),       # absolute only
]


def _case(name, rule, w, clone, core, copies, cand=None):
    return dict(name=name, rule=rule, w=w, clone=clone, core=core, copies=copies, cand=cand or {})


def cases():
    out = []
    # S3: duplicates need equal length, bitsets and bytes; the representative
    # is the minimum row index and copies[rep] = class size
    # (cuda/PSDBSCAN.hcu:525-573, 76-107, 1074-1085).  Hamming eps=0: no neighbours.
    w = from_strings([b"CAR", b"CAK", b"CAR", b"CAR", b"CAK", b"GG"], None, None, [], [],
                     abs_eps=0, min_pts=3, use_hamming=True)
    out.append(_case("dup_classes", "S3", w, clone=[1, 0, 1, 1, 0, 0], core=[1, 0, 0, 0, 0, 0],
                     copies=[3, 2, 0, 0, 0, 1]))
    # S4/S5/S7 Hamming mode, eps=1, minPts=2.  d(0,1)=1, d(1,2)=1, d(0,2)=2,
    # d(2,3)=2, GGGG is 4 from all.  counts: 0:2+1=3, 1:1+2+1=4, 2:1+1=2, 3:1, 5:1.
    w = from_strings([b"AAAA", b"AAAC", b"AACC", b"CCCC", b"AAAA", b"GGGG"], None, None, [], [],
                     abs_eps=1, min_pts=2, use_hamming=True)
    out.append(_case("hamming_chain", "S4 S5 S6 S7", w, clone=[1, 1, 1, 0, 1, 0],
                     core=[1, 1, 1, 0, 0, 0], copies=[2, 1, 1, 1, 0, 1]))
    # S5: a duplicate class with copies >= minPts is core without neighbours.
    w = from_strings([b"AAAA", b"AAAA", b"AAAA", b"CCCC"], None, None, [], [], abs_eps=1,
                     min_pts=3, use_hamming=True)
    out.append(_case("copies_core", "S5", w, clone=[1, 1, 1, 0], core=[1, 0, 0, 0],
                     copies=[3, 0, 0, 1]))
    # S6: border row 2 touches the cores of two clusters (0 and 1, distance 2
    # apart).  minPts=4: x1 and x2 have 4 neighbours each (count 5), y has 2
    # (count 3).  Deterministic rule: the minimum-index core neighbour (row 0,
    # cluster 1); the reference's race allows clusters {1, 2}.
    seqs = [b"AAAAA", b"CAAAC", b"AAAAC", b"GAAAA", b"TAAAA", b"AGAAA", b"CAAGC", b"CAATC",
            b"CATAC"]
    w = from_strings(seqs, None, None, [], [], abs_eps=1, min_pts=4, use_hamming=True)
    out.append(_case("border_two_clusters", "S6", w, clone=[1, 2, 1, 1, 1, 1, 2, 2, 2],
                     core=[1, 1, 0, 0, 0, 0, 0, 0, 0], copies=[1] * 9, cand={2: [1, 2]}))
    # S1+S3+S4: equal sequences with disjoint V sets are neither duplicates nor
    # neighbours; a row whose V set overlaps both links them; a call matching no
    # gene gives a zero bitset, compatible with nobody.
    w = from_strings([b"CARDY"] * 4,
                     [b"IGHV1-2*01", b"IGHV3-23*01", b"IGHV1-2*01, or IGHV3-23*01", b"IGHV9-9*01"],
                     [b"IGHJ4*02"] * 4, V3, [b"IGHJ4*"], abs_eps=1, min_pts=2, use_hamming=True)
    out.append(_case("vj_overlap", "S1 S3 S4", w, clone=[1, 1, 1, 0], core=[1, 1, 1, 0],
                     copies=[1, 1, 1, 1]))
    # S4 Levenshtein mode with the relative threshold t=0.2:
    # eps(10,9)=2, eps(10,10)=2, eps(12,10)=2, eps(12,9)=2 (gap 3 > 2).
    # lev(0,1)=1, lev(0,2)=2 (Hamming 7), lev(0,4)=2, lev(2,4)=2, lev(1,2)=3.
    w = from_strings([b"ACDEFGHIKL", b"ACDEFGHIK", b"ACDFGHIKLM", b"MMMMMMMMMM",
                      b"ACDEFGHIKLMN"], None, None, [], [], threshold=0.2, min_pts=2,
                     use_hamming=False)
    out.append(_case("levenshtein_relative", "S2 S4", w, clone=[1, 1, 1, 0, 1],
                     core=[1, 1, 1, 0, 1], copies=[1, 1, 1, 1, 1]))
    # Same rows in Hamming mode: only equal lengths compare; all far apart.
    w = from_strings([b"ACDEFGHIKL", b"ACDEFGHIK", b"ACDFGHIKLM", b"MMMMMMMMMM",
                      b"ACDEFGHIKLMN"], None, None, [], [], threshold=0.2, min_pts=2,
                     use_hamming=True)
    out.append(_case("hamming_relative", "S4", w, clone=[0] * 5, core=[0] * 5, copies=[1] * 5))
    # minPts = 1: every unique is core; duplicates are not (count 0, :1099).
    w = from_strings([b"AAA", b"AAA", b"CCC"], None, None, [], [], abs_eps=0, min_pts=1,
                     use_hamming=True)
    out.append(_case("minpts1", "S5 S7", w, clone=[1, 1, 2], core=[1, 0, 1], copies=[2, 0, 1]))
    # minPts = 0: duplicates are core too (0 >= 0, :1180).
    w = from_strings([b"AAA", b"AAA", b"CCC"], None, None, [], [], abs_eps=0, min_pts=0,
                     use_hamming=True)
    out.append(_case("minpts0", "S5 S7", w, clone=[1, 1, 2], core=[1, 1, 1], copies=[2, 0, 1]))
    # Independent repertoires: no duplicates or neighbours across them, labels
    # restart at 1.
    w = from_strings([b"AAAA", b"AAAC", b"AAAA", b"AAAC"], None, None, [], [], abs_eps=1,
                     min_pts=2, use_hamming=True, rep_sizes=[2, 2])
    out.append(_case("repertoires", "S7", w, clone=[1, 1, 1, 1], core=[1, 1, 1, 1],
                     copies=[1, 1, 1, 1]))
    # Labels are numbered by ascending minimum core row (:1274-1286): the cluster
    # whose first core row is 0 gets 1 even though its other members come later.
    w = from_strings([b"GGGG", b"AAAA", b"AAAC", b"GGGT", b"TTTT"], None, None, [], [],
                     abs_eps=1, min_pts=2, use_hamming=True)
    out.append(_case("label_order", "S7", w, clone=[1, 2, 2, 1, 0], core=[1, 1, 1, 1, 0],
                     copies=[1] * 5))
    return out


def no_seq_case():
    """No sequence column: every row is "Gene" (cpp/TableHolder.hpp:326-328)."""
    w = from_strings([b"Gene"] * 3, [b"IGHV1-2*01", b"IGHV1-2*01", b"IGHV3-23*01"], None, V3, [],
                     abs_eps=1, min_pts=2, use_hamming=True)
    return w, dict(clone=[1, 1, 0], core=[1, 0, 0], copies=[2, 0, 1])
