"""Parity at the benchmarked sizes: the library against the oracle's indexed mode
(the all-pairs answer; tests/test_oracle.py checks the two modes agree) on whole
workloads or large fractions of them, including the reference's own relative
threshold (maximum_relative_edit_distance, cuda/SpecialFunctors.hcu:257-261) in
Hamming mode, where eps varies with the length and the segment join runs with
a segment count per length.  Bit-exact: clone ids, core flags, copies."""
import numpy as np
import pytest

import oracle
from immunodbscan_gb300 import cluster_workload, synth
from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


def _check(gpu_ctx, w, label, candidates=None):
    g = cluster_workload(w, gpu_ctx)
    o = oracle.cluster(w, indexed=True)
    assert_same(g, o, w, label)
    assert g.stats.neighbour_pairs == o.neighbour_pairs, label
    assert g.stats.n_clusters == o.n_clusters, label
    if candidates is not None:
        assert g.stats.candidates == candidates, label
    return g


def test_workload1_full_size(gpu_ctx):
    """200,000 nucleotide CDR3s, Levenshtein eps=2, minPts=3 (every row)."""
    w = synth.workload(1)
    assert w.n == 200_000
    _check(gpu_ctx, w, "workload1 full")


@pytest.mark.parametrize("threshold,join", [(0.1, 1), (0.15, 0)])
def test_hamming_relative_threshold_workload0_full(gpu_ctx, threshold, join):
    """10,000 amino-acid CDR3s of length 8-25 with no absolute eps: eps =
    trunc(0.1 L) is 0-2 (segment join, per-length segment counts) and
    trunc(0.15 L) reaches 3 (buckets)."""
    w = synth.workload(0)
    w.abs_eps, w.threshold = -1, threshold
    _check(gpu_ctx, w, f"workload0 t={threshold}", candidates=join)


@pytest.mark.parametrize("threshold,join", [(0.1, 1), (0.15, 0)])
def test_hamming_relative_threshold_workload2(gpu_ctx, threshold, join):
    """The 64-repertoire workload at 6% (about 300k rows) with the relative
    threshold only."""
    w = synth.workload(2, scale=0.06)
    w.abs_eps, w.threshold = -1, threshold
    _check(gpu_ctx, w, f"workload2@0.06 t={threshold}", candidates=join)


def test_workload2_ten_percent(gpu_ctx):
    """The bench workload's rule (Hamming eps=1) on 10% of its rows."""
    w = synth.workload(2, scale=0.1)
    _check(gpu_ctx, w, "workload2@0.1", candidates=1)


def test_workload3_100k(gpu_ctx):
    """V/J usage Zipf(1.8), Levenshtein eps=2, 100,000 rows."""
    w = synth.workload(3, scale=0.05)
    assert w.n >= 100_000
    _check(gpu_ctx, w, "workload3@0.05")


def test_workload4_200k(gpu_ctx):
    """Lengths Normal(16,3.5), eps = min(3, trunc(0.15 L)), minPts=4, 200,000 rows."""
    w = synth.workload(4, scale=0.02)
    assert w.n >= 200_000
    _check(gpu_ctx, w, "workload4@0.02")


def test_workload4_relative_only(gpu_ctx):
    """Workload 4's rows with the reference's key alone (threshold 0.15, no cap)."""
    w = synth.workload(4, scale=0.01)
    w.abs_eps = -1
    _check(gpu_ctx, w, "workload4@0.01 relative")
