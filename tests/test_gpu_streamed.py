"""Streamed mode: when the neighbour-pair list may not take the memory it needs
(idb_params.edge_memory_mb), the pairs are not stored and the distance work runs
twice -- a counting sweep, then a sweep that merges core-core pairs and keeps
each non-core unique's minimum core neighbour.  The answer must be the edge-list
path's, bit for bit, for every candidate path (segment join, buckets,
Levenshtein), forced from the start (edge_memory_mb < 0) or switched to after
the first sweep overflows a small budget, eagerly and under a captured plan."""
import dataclasses

import numpy as np
import pytest

import oracle
from immunodbscan_gb300 import DeviceBatch, cluster_workload, synth

pytestmark = pytest.mark.gpu

CASES = [
    ("join", lambda: synth.workload(2, scale=0.01)),
    ("join_large", lambda: synth.workload(2, scale=0.1)),
    ("buckets", lambda: dataclasses.replace(synth.workload(2, scale=0.01), candidates=1)),
    ("levenshtein", lambda: synth.workload(3, scale=0.01)),
    ("levenshtein_minpts4", lambda: synth.workload(4, scale=0.003)),
    ("nt_levenshtein", lambda: synth.workload(1, scale=0.02)),
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("budget_mb", [-1, 1])
def test_streamed_matches_edge_list(gpu_ctx, name, make, budget_mb):
    w = make()
    base = cluster_workload(w, gpu_ctx, eval_trees=True)
    assert base.stats.streamed == 0
    ws = dataclasses.replace(w, edge_memory_mb=budget_mb)
    got = cluster_workload(ws, gpu_ctx, eval_trees=True)
    # the list takes 8 bytes a pair: past 1 MiB the first sweep overflows it
    if budget_mb < 0 or base.stats.neighbour_pairs * 8 > (1 << 20):
        assert got.stats.streamed == 1, name
    assert np.array_equal(got.copies, base.copies), name
    assert np.array_equal(got.core, base.core), name
    assert np.array_equal(got.clone_id, base.clone_id), name
    assert got.stats.neighbour_pairs == base.stats.neighbour_pairs
    assert got.stats.n_clusters == base.stats.n_clusters
    # rows that are their own root and the histogram's total do not depend on
    # how the forest was built
    assert int(got.tree_depth_hist[0]) == int(base.tree_depth_hist[0])
    assert int(got.tree_depth_hist.sum()) == w.n


def test_streamed_matches_oracle_and_replays(gpu_ctx):
    w = dataclasses.replace(synth.workload(2, scale=0.01), edge_memory_mb=-1)
    o = oracle.cluster(w)
    b = DeviceBatch(w, gpu_ctx)
    b.plan()
    for _ in range(2):
        st = b.run()
        assert st.streamed == 1
        clone, core, copies = b.results()
        assert np.array_equal(clone, o.clone_id)
        assert np.array_equal(core, o.core)
        assert np.array_equal(copies, o.copies)
