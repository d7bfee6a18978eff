"""GPU path (libimmunodbscan_gb300 through the C ABI) against the oracle.

Integer work throughout, so the bar is bit-exact: clone ids, core flags and
copies identical to the oracle (both use the minimum-index core neighbour for
border rows), plus the reference-semantics check that every border label is one
of the clusters the reference's first-wins race could have produced.
"""
import math

import numpy as np
import pytest

import oracle
from immunodbscan_gb300 import DeviceBatch, IdbError, cluster_workload, synth
from kat_cases import cases, no_seq_case

pytestmark = pytest.mark.gpu


def assert_same(gpu, ora, w, label=""):
    assert np.array_equal(gpu.copies, ora.copies), f"{label}: copies differ"
    assert np.array_equal(gpu.core, ora.core), f"{label}: core flags differ"
    bad = np.nonzero(gpu.clone_id != ora.clone_id)[0]
    assert bad.size == 0, (f"{label}: {bad.size} clone ids differ, first rows {bad[:8].tolist()} "
                           f"gpu={gpu.clone_id[bad[:8]].tolist()} ora={ora.clone_id[bad[:8]].tolist()}")
    assert gpu.n_uniques == ora.n_uniques
    # reference semantics: a border row may carry any of its core neighbours' clusters
    K = ora.cand.shape[1]
    for i in np.nonzero(ora.n_cand > 1)[0][:2000]:
        nc = int(ora.n_cand[i])
        if nc <= K:
            assert int(gpu.clone_id[i]) in ora.cand[i, :nc].tolist()


@pytest.mark.parametrize("case", cases(), ids=lambda c: c["name"])
def test_known_answers(gpu_ctx, case):
    r = cluster_workload(case["w"], gpu_ctx)
    assert r.clone_id.tolist() == case["clone"]
    assert r.core.tolist() == case["core"]
    assert r.copies.tolist() == case["copies"]


def test_no_sequence_column(gpu_ctx):
    w, want = no_seq_case()
    r = cluster_workload(w, gpu_ctx, no_seq=True)
    assert r.clone_id.tolist() == want["clone"]
    assert r.core.tolist() == want["core"]
    assert r.copies.tolist() == want["copies"]


@pytest.mark.parametrize("k,scale", [(0, 1.0), (0, 0.2), (1, 0.03), (2, 0.004), (3, 0.01),
                                     (4, 0.0015)])
def test_workloads_vs_oracle(gpu_ctx, k, scale):
    w = synth.workload(k, scale=scale)
    g = cluster_workload(w, gpu_ctx)
    o = oracle.cluster(w)
    assert_same(g, o, w, f"workload{k}@{scale}")
    assert g.stats.neighbour_pairs == o.neighbour_pairs
    assert g.stats.n_clusters == o.n_clusters


@pytest.mark.parametrize("k", [1, 3, 4])
def test_relative_threshold_only(gpu_ctx, k):
    w = synth.workload(k, scale=0.004 if k != 4 else 0.001)
    w.abs_eps = -1
    w.threshold = 0.15
    g = cluster_workload(w, gpu_ctx)
    o = oracle.cluster(w)
    assert_same(g, o, w, f"relative{k}")


@pytest.mark.parametrize("hamming", [True, False])
def test_no_gene_columns(gpu_ctx, hamming):
    w = synth.workload(0, scale=0.1)
    w.use_hamming = hamming
    g = cluster_workload(w, gpu_ctx, no_v=True, no_j=True)
    o = oracle.cluster(w, no_v=True, no_j=True)
    assert_same(g, o, w, "no genes")


def _random_workload(rng, n, lo, hi, alphabet, hamming, eps, min_pts, n_fam=None):
    fam = n_fam or max(n // 8, 1)
    roots = [rng.choice(alphabet, size=int(rng.integers(lo, hi + 1))).astype(np.uint8).tobytes()
             for _ in range(fam)]
    seqs = []
    for i in range(n):
        s = bytearray(roots[int(rng.integers(0, fam))])
        for _ in range(int(rng.poisson(1.0))):
            p = int(rng.integers(0, len(s)))
            s[p] = int(rng.choice(alphabet))
        if not hamming and rng.random() < 0.2 and len(s) > lo:
            del s[int(rng.integers(0, len(s)))]
        seqs.append(bytes(s))
    vg = [b"IGHV%d*" % g for g in range(1, 9)]
    jg = [b"IGHJ%d*" % g for g in range(1, 4)]
    vc = [b"IGHV%d*01, or IGHV%d*01" % (1 + rng.integers(0, 8), 1 + rng.integers(0, 8))
          for _ in range(n)]
    jc = [b"IGHJ%d*02" % (1 + rng.integers(0, 3)) for _ in range(n)]
    return synth.from_strings(seqs, vc, jc, vg, jg, abs_eps=eps, min_pts=min_pts,
                              use_hamming=hamming)


@pytest.mark.parametrize("hamming", [True, False])
def test_wide_gene_lists(gpu_ctx, hamming):
    """More than 64 V genes and more than 32 J genes: multi-word bitsets, and a
    neighbour's canonical bin is decided from the full bitsets (lowest common V
    and J gene) instead of the one-word signatures; ambiguous calls of 1-4
    genes spread each unique over many bins, small and large."""
    rng = np.random.default_rng(21)
    n = 6000
    w0 = _random_workload(rng, n, 10, 16, list(b"ACDEFGHIKLMNPQRSTVWY"), hamming, 1, 2,
                          n_fam=300)
    vg = [b"TRBV%d-%d*" % (a, b) for a in range(1, 31) for b in range(1, 6)]     # 150
    jg = [b"TRBJ%d-%d*" % (a, b) for a in range(1, 9) for b in range(1, 6)]      # 40
    seqs = [w0.seq(i) for i in range(n)]
    vc, jc = [], []
    for s in seqs:
        # a length-dependent gene shared by most neighbours, plus random extras
        gv = {(len(s) // 3) * 7 % len(vg)} | set(rng.choice(len(vg), size=int(rng.integers(0, 4))).tolist())
        gj = {(len(s) // 4) * 5 % len(jg)} | set(rng.choice(len(jg), size=int(rng.integers(0, 3))).tolist())
        vc.append(b", or ".join(vg[g][:-1] + b"*01" for g in sorted(gv)))
        jc.append(b", or ".join(jg[g][:-1] + b"*01" for g in sorted(gj)))
    w = synth.from_strings(seqs, vc, jc, vg, jg, abs_eps=1, min_pts=2, use_hamming=hamming)
    assert_same(cluster_workload(w, gpu_ctx), oracle.cluster(w), w, "wide gene lists")


@pytest.mark.parametrize("hamming", [True, False])
@pytest.mark.parametrize("lo,hi", [(30, 40), (60, 70), (90, 128)])
def test_multiword_lengths(gpu_ctx, hamming, lo, hi):
    rng = np.random.default_rng(lo + hamming)
    w = _random_workload(rng, 1500, lo, hi, list(b"ACDEFGHIKLMNPQRSTVWY"), hamming, 3, 2)
    g = cluster_workload(w, gpu_ctx)
    o = oracle.cluster(w)
    assert_same(g, o, w, f"multiword {lo}-{hi}")


@pytest.mark.parametrize("hamming", [True, False])
def test_generic_alphabet(gpu_ctx, hamming):
    """More than 32 distinct byte values: the generic (byte) kernels."""
    rng = np.random.default_rng(7)
    w = _random_workload(rng, 1200, 10, 20, list(range(33, 127)), hamming, 2, 2)
    g = cluster_workload(w, gpu_ctx)
    o = oracle.cluster(w)
    assert_same(g, o, w, "generic alphabet")


@pytest.mark.parametrize("hamming", [True, False])
def test_generic_long(gpu_ctx, hamming):
    """Sequences longer than 128: the generic kernels (Levenshtein up to 1024)."""
    rng = np.random.default_rng(11)
    w = _random_workload(rng, 400, 150, 300, list(b"ACGT"), hamming, 6, 2, n_fam=40)
    g = cluster_workload(w, gpu_ctx)
    o = oracle.cluster(w)
    assert_same(g, o, w, "generic long")


@pytest.mark.parametrize("eps", [0, 1, 2, 3])
@pytest.mark.parametrize("lo,hi", [(1, 7), (6, 24), (40, 70)])
def test_segment_join(gpu_ctx, eps, lo, hi):
    """Hamming with eps <= 2 at every length: candidates come from the segment
    join (eps 3: the buckets, same answers).  Short sequences (fewer residues
    than segments: empty segments), identical sequences under different gene
    calls (identical in every segment, emitted from the lowest), disjoint V or
    J sets (rejected at the hit) and a small alphabet (large groups) against
    the oracle."""
    rng = np.random.default_rng(100 * eps + lo)
    w0 = _random_workload(rng, 3000, lo, hi, list(b"ACGT"), True, eps, 2, n_fam=120)
    seqs = [w0.seq(i) for i in range(w0.n)]
    seqs += [seqs[int(i)] for i in rng.integers(0, len(seqs), size=600)]
    vg = [b"IGHV%d*" % g for g in range(1, 9)]
    jg = [b"IGHJ%d*" % g for g in range(1, 4)]
    vc = [b"IGHV%d*01" % (1 + rng.integers(0, 8)) for _ in seqs]
    jc = [b"IGHJ%d*02, or IGHJ%d*01" % (1 + rng.integers(0, 3), 1 + rng.integers(0, 3))
          for _ in seqs]
    w = synth.from_strings(seqs, vc, jc, vg, jg, abs_eps=eps, min_pts=2, use_hamming=True)
    g = cluster_workload(w, gpu_ctx)
    o = oracle.cluster(w)
    assert_same(g, o, w, f"segment join eps={eps} L={lo}-{hi}")
    assert g.stats.neighbour_pairs == o.neighbour_pairs
    assert g.stats.candidates == (1 if eps <= 2 else 0)


def test_nucleotide_two_planes(gpu_ctx):
    w = synth.workload(1, scale=0.02)
    w.use_hamming = True
    g = cluster_workload(w, gpu_ctx)
    o = oracle.cluster(w)
    assert_same(g, o, w, "nt hamming")


def test_deterministic_and_stats(gpu_ctx):
    w = synth.workload(3, scale=0.01)
    a = cluster_workload(w, gpu_ctx)
    b = cluster_workload(w, gpu_ctx)
    assert np.array_equal(a.clone_id, b.clone_id)
    assert a.stats.n_uniques == b.stats.n_uniques
    assert a.stats.pairs_evaluated == b.stats.pairs_evaluated
    assert a.stats.pairs_evaluated >= a.stats.neighbour_pairs


def test_tree_depth_histogram(gpu_ctx):
    w = synth.workload(0, scale=0.3)
    r = cluster_workload(w, gpu_ctx, eval_trees=True)
    assert r.tree_depth_hist is not None
    assert int(r.tree_depth_hist.sum()) == w.n


def test_uniques_getter(gpu_ctx):
    w = synth.workload(0, scale=0.1)
    r = cluster_workload(w, gpu_ctx)
    want = np.nonzero(r.copies)[0]
    assert np.array_equal(r.uniques[: r.n_uniques], want)


def test_empty_and_single(gpu_ctx):
    w = synth.from_strings([], None, None, [], [], abs_eps=1, min_pts=2, use_hamming=True)
    r = cluster_workload(w, gpu_ctx)
    assert r.clone_id.size == 0
    w = synth.from_strings([b"CARDY"], None, None, [], [], abs_eps=1, min_pts=1, use_hamming=True)
    r = cluster_workload(w, gpu_ctx)
    assert r.clone_id.tolist() == [1] and r.core.tolist() == [1] and r.copies.tolist() == [1]


def test_invalid_arguments(gpu_ctx):
    w = synth.workload(0, scale=0.01)
    w.abs_eps = -1
    w.threshold = math.nan
    with pytest.raises(IdbError) as e:
        cluster_workload(w, gpu_ctx)
    assert e.value.status == 1


def test_batch_graph_matches_plain(gpu_ctx):
    w = synth.workload(2, scale=0.003)
    plain = cluster_workload(w, gpu_ctx)
    b = DeviceBatch(w, gpu_ctx)
    b.plan()
    for _ in range(2):
        st = b.run()
        clone, core, copies = b.results()
        assert np.array_equal(clone, plain.clone_id)
        assert np.array_equal(core, plain.core)
        assert np.array_equal(copies, plain.copies)
        assert st.n_uniques == plain.stats.n_uniques


def test_device_api_matches_host_api(gpu_ctx):
    w = synth.workload(1, scale=0.01)
    plain = cluster_workload(w, gpu_ctx)
    b = DeviceBatch(w, gpu_ctx)
    b.cluster_once()
    clone, core, copies = b.results()
    assert np.array_equal(clone, plain.clone_id)
    assert np.array_equal(copies, plain.copies)


def _gpu_bits(ctx, calls, genes):
    import ctypes as C
    from immunodbscan_gb300 import _lib
    from immunodbscan_gb300.interlink import _as_blob
    cb, co = _as_blob(calls)
    gb, go = _as_blob(genes)
    W = max(1, (len(genes) + 63) // 64)
    out = np.zeros((len(calls), W), np.uint64)
    _lib.check(_lib.lib().idb_diag_gene_bits(ctx.handle, cb.ctypes.data, co.ctypes.data,
                                             len(calls), gb.ctypes.data, go.ctypes.data,
                                             len(genes), out.ctypes.data))
    return out


def _as_words32(bits64, n_genes):
    w32 = (n_genes + 31) // 32
    out = np.zeros((bits64.shape[0], w32), np.uint32)
    for k in range(w32):
        out[:, k] = (bits64[:, k // 2] >> np.uint64(32 * (k % 2))) & np.uint64(0xFFFFFFFF)
    return out


def test_gene_bits_known_answers(gpu_ctx):
    from kat_cases import S1_CALLS, S1_GENES, S1_WORDS
    got = _as_words32(_gpu_bits(gpu_ctx, S1_CALLS, S1_GENES), len(S1_GENES))
    assert got.tolist() == S1_WORDS


GENE_BIT_MODES = ["short", "long_calls", "long_names", "huge_calls", "repeated"]


@pytest.mark.parametrize("mode", GENE_BIT_MODES)
def test_gene_bits_vs_oracle(gpu_ctx, mode):
    """Random names (incl. empty, repeated, overlapping and prefix-sharing ones)
    against random calls.  Long calls fill a warp's staging slice after fewer than
    32 rows; a call longer than the slice (huge_calls) or a name longer than 255
    bytes takes the per-row path; repeated calls share a representative row."""
    rng = np.random.default_rng(5 + GENE_BIT_MODES.index(mode))
    alpha = list(b"ACGT*-I0123")
    genes = [bytes(rng.choice(alpha, size=int(rng.integers(1, 7))).astype(np.uint8)) for _ in range(150)]
    genes += [b"", genes[3], genes[7] + b"*"] + ([b"A" * 300] if mode == "long_names" else [])
    calls = []
    for i in range(3000):
        if mode == "repeated" and i >= 40:
            calls.append(calls[int(rng.integers(0, 40))])
            continue
        if mode == "huge_calls":
            n = int(rng.integers(2040, 3000)) if i % 100 == 3 else int(rng.integers(0, 60))
        else:
            n = int(rng.integers(0, 60 if mode in ("short", "repeated") else
                                 (400 if i % 200 < 40 else 30)))
        s = bytearray(rng.choice(alpha, size=n).astype(np.uint8).tobytes())
        if rng.random() < 0.5 and n > 10:
            g = genes[int(rng.integers(0, len(genes)))]
            p = int(rng.integers(0, n))
            s[p:p] = g
        calls.append(bytes(s))
    got = _as_words32(_gpu_bits(gpu_ctx, calls, genes), len(genes))
    want = oracle.gene_bitsets(calls, genes)
    assert np.array_equal(got, want)


def test_gene_bits_call_table_overflow(gpu_ctx):
    """More distinct calls than the call-string table holds (2^20 slots): rows
    that find no slot compute their own bitsets."""
    rng = np.random.default_rng(9)
    n = 1_200_000
    genes = [b"IGHV%d" % k for k in range(1, 70)] + [b"-1", b"*0"]
    # distinct calls: a gene name plus a unique decimal suffix; some repeated
    idx = rng.integers(0, 69, size=n)
    calls = [b"IGHV%d-%d*0%d" % (idx[i] + 1, i, i % 7) for i in range(n)]
    for i in range(0, n, 1000):
        calls[i] = calls[i // 2]
    got = _as_words32(_gpu_bits(gpu_ctx, calls, genes), len(genes))
    assert np.array_equal(got, oracle.gene_bitsets(calls, genes))


def test_gene_bits_synthetic(gpu_ctx):
    w = synth.workload(2, scale=0.002)
    calls = [w.vcall(i) for i in range(w.n)]
    got = _as_words32(_gpu_bits(gpu_ctx, calls, w.v_genes), len(w.v_genes))
    assert np.array_equal(got, oracle.gene_bitsets(calls, w.v_genes))


def test_candidates_buckets_same_partition(gpu_ctx):
    """idb_params.candidates = 1 scores every admissible pair of the buckets
    instead of the segment join; the answer is the same."""
    w = synth.workload(2, scale=0.004)
    g0 = cluster_workload(w, gpu_ctx)
    w.candidates = 1
    g1 = cluster_workload(w, gpu_ctx)
    assert g0.stats.candidates == 1 and g1.stats.candidates == 0
    assert g1.stats.pairs_evaluated > g0.stats.pairs_evaluated
    assert g0.stats.neighbour_pairs == g1.stats.neighbour_pairs
    assert np.array_equal(g0.clone_id, g1.clone_id)
    assert np.array_equal(g0.core, g1.core)
    assert np.array_equal(g0.copies, g1.copies)


import ref_fixtures  # noqa: E402


@pytest.mark.parametrize("name", ref_fixtures.names())
def test_reference_fixtures(gpu_ctx, name):
    """The library against the reference's own answers (its InterlinkClass on
    the same rows): clone ids, cores, copies, uniques, and the parts of the
    tree-depth histogram that do not depend on the union order."""
    _, w, want = next(c for c in ref_fixtures.load() if c[0] == name)
    r = cluster_workload(w, gpu_ctx, eval_trees=True)
    ref_fixtures.assert_matches(name, want, r.clone_id, r.core, r.copies,
                                uniques=r.uniques[: r.n_uniques], hist=r.tree_depth_hist)
