"""Host columns copied and pre-processed by row chunks (idb_params.row_chunks):
the gene-bitset and duplicate kernels of chunk k run while later chunks are
still being copied.  Every chunk count gives the oracle's answer, on the eager
path, on the call that captures the shape and on replays of it (whose graph
waits on the copy events of its own call), with absent gene columns, and at
2^20+ rows where the chunks are chosen automatically."""
import dataclasses

import numpy as np
import pytest

import oracle
from immunodbscan_gb300 import Context, cluster_workload, synth

pytestmark = pytest.mark.gpu


def _same(g, o, label):
    assert np.array_equal(g.copies, o.copies), label
    assert np.array_equal(g.core, o.core), label
    assert np.array_equal(g.clone_id, o.clone_id), label


@pytest.mark.parametrize("chunks", [1, 2, 3, 8])
def test_chunk_counts_match_oracle(chunks):
    w = synth.workload(2, scale=0.004)
    w.row_chunks = chunks
    o = oracle.cluster(w)
    with Context(0) as ctx:
        for k in range(4):   # eager, eager + capture, replays
            _same(cluster_workload(w, ctx), o, f"{chunks} chunks, call {k}")


@pytest.mark.parametrize("no_v,no_j", [(True, False), (False, True), (True, True)])
def test_chunks_with_absent_gene_columns(no_v, no_j):
    w = synth.workload(0, scale=0.5)
    w.row_chunks = 5
    o = oracle.cluster(w, no_v=no_v, no_j=no_j)
    with Context(0) as ctx:
        for k in range(3):
            _same(cluster_workload(w, ctx, no_v=no_v, no_j=no_j), o, f"call {k}")


def test_chunks_levenshtein_and_new_data_on_replay():
    """Levenshtein rows in 7 chunks; later calls of the shape bring new rows
    (a replay must copy and wait for this call's columns, not reuse the last)."""
    w = synth.workload(1, scale=0.02)
    w.row_chunks = 7
    rng = np.random.default_rng(5)
    with Context(0) as ctx:
        for k in range(5):
            perm = rng.permutation(w.n) if k else np.arange(w.n)
            wk = synth.take_rows(w, perm)
            wk = dataclasses.replace(wk, row_chunks=7)
            g = cluster_workload(wk, ctx)
            _same(g, oracle.cluster(wk), f"call {k}")


def test_automatic_chunks_above_a_million_rows():
    """1.1M rows (64 repertoires, Hamming eps=1): eight chunks by default."""
    w = synth.workload(2, scale=0.22)
    assert w.n >= 1 << 20
    o = oracle.cluster(w, indexed=True)
    with Context(0) as ctx:
        for k in range(3):
            _same(cluster_workload(w, ctx), o, f"call {k}")
        w1 = dataclasses.replace(w, row_chunks=1)
        _same(cluster_workload(w1, ctx), o, "one chunk")


def test_chunks_number_uniques_in_row_order():
    """Unique ids ascend with the representative row whatever the chunking:
    the uniques output lists the rows with copies > 0 in order, and the
    row -> unique map agrees with it."""
    w = synth.workload(2, scale=0.006)
    with Context(0) as ctx:
        ref = None
        for chunks in (1, 3, 8):
            w.row_chunks = chunks
            r = cluster_workload(w, ctx)
            reps = np.nonzero(r.copies > 0)[0]
            assert r.n_uniques == reps.size, chunks
            assert np.array_equal(np.asarray(r.uniques[: r.n_uniques]), reps), chunks
            if ref is None:
                ref = r
            _same(r, ref, f"{chunks} chunks against 1")


def test_chunks_with_streamed_mode_and_tree_depths():
    """Row chunks with no neighbour-pair list (streamed mode), and with the
    tree-depth histogram (its total and bin 0 do not depend on the order of
    the unions)."""
    w = synth.workload(2, scale=0.004)
    o = oracle.cluster(w)
    with Context(0) as ctx:
        w.row_chunks, w.edge_memory_mb = 5, -1
        g = cluster_workload(w, ctx)
        assert g.stats.streamed == 1
        _same(g, o, "streamed, 5 chunks")
        w.edge_memory_mb = 0
        h1 = cluster_workload(dataclasses.replace(w, row_chunks=1), ctx, eval_trees=True).tree_depth_hist
        h5 = cluster_workload(w, ctx, eval_trees=True).tree_depth_hist
        assert int(np.sum(h1)) == int(np.sum(h5)) == w.n
        assert int(h1[0]) == int(h5[0])
