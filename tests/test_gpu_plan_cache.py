"""idb_cluster's plan cache: the second call of an input shape captures its launch
sequence and later calls of that shape replay it.  A replay must give the eager
answer for new data of the same shape, fall back to the eager path when the
data leaves the plan (new byte values, longer sequences, more neighbour pairs
than the captured capacities), and never replay across a call of another
shape.  A batch plan whose staged inputs another call replaced is refused."""
import dataclasses

import numpy as np
import pytest

import oracle
from immunodbscan_gb300 import Context, DeviceBatch, IdbError, cluster_workload, synth

pytestmark = pytest.mark.gpu


def _mutated(w, seed, *, new_byte=None, longer=False, collapse=False):
    """Same rows, gene calls and repertoires; sequences changed in place."""
    rng = np.random.default_rng(seed)
    seqs = [bytearray(w.seq(i)) for i in range(w.n)]
    alpha = sorted(set(w.seq_blob.tolist()))
    for s in seqs:
        if s and rng.random() < 0.3:
            s[int(rng.integers(0, len(s)))] = int(rng.choice(alpha))
    if new_byte is not None:
        seqs[w.n // 2][0] = new_byte
    if longer:
        seqs[w.n // 3] += b"A" * 40
    if collapse:   # every row of a repertoire one of two sequences: dense neighbourhoods
        for r in range(w.n_rep):
            lo, hi = int(w.rep_off[r]), int(w.rep_off[r + 1])
            for i in range(lo, hi):
                seqs[i] = bytearray(b"CARDYW" if i % 2 else b"CARDYF")
    off = np.zeros(w.n + 1, np.int64)
    np.cumsum([len(s) for s in seqs], out=off[1:])
    blob = np.frombuffer(b"".join(bytes(s) for s in seqs), np.uint8).copy()
    return dataclasses.replace(w, seq_blob=blob, seq_off=off)


def _same(g, o, label):
    assert np.array_equal(g.copies, o.copies), label
    assert np.array_equal(g.core, o.core), label
    assert np.array_equal(g.clone_id, o.clone_id), label


def test_replay_matches_eager_and_falls_back():
    w = synth.workload(2, scale=0.004)
    with Context(0) as ctx:
        r1 = cluster_workload(w, ctx)              # eager
        r2 = cluster_workload(w, ctx)              # eager, then capture
        r3 = cluster_workload(w, ctx)              # replay
        assert r1.stats.kernel_launches == 0 and r3.stats.kernel_launches > 0
        for r in (r2, r3):
            _same(r, r1, "same data")
        assert r3.n_uniques == r1.n_uniques
        assert np.array_equal(r3.uniques[: r3.n_uniques], r1.uniques[: r1.n_uniques])
        # new data of the same shape: replayed
        for seed in (1, 2):
            wm = _mutated(w, seed)
            g = cluster_workload(wm, ctx)
            assert g.stats.kernel_launches > 0, "expected a replay"
            _same(g, oracle.cluster(wm), f"mutated {seed}")
        # data outside the plan: a byte value never seen, a longer sequence,
        # far more neighbour pairs -- eager fallback, same answer as the oracle
        for kw in ({"new_byte": ord("#")}, {"longer": True}, {"collapse": True}):
            wm = _mutated(w, 3, **kw)
            _same(cluster_workload(wm, ctx), oracle.cluster(wm), f"outside the plan {kw}")


def test_no_replay_across_shapes():
    wa = synth.workload(2, scale=0.003)
    wb = synth.workload(0, scale=0.2)
    oa, ob = oracle.cluster(wa), oracle.cluster(wb)
    with Context(0) as ctx:
        for w, o in [(wa, oa), (wa, oa), (wb, ob), (wa, oa), (wa, oa), (wb, ob), (wb, ob),
                     (wa, oa), (wb, ob), (wb, ob), (wb, ob)]:
            _same(cluster_workload(w, ctx), o, w.name)


def test_batch_plan_refused_after_other_call():
    w = synth.workload(2, scale=0.003)
    with Context(0) as ctx:
        b = DeviceBatch(w, ctx)
        b.plan()
        b.run()
        cluster_workload(synth.workload(0, scale=0.1), ctx)   # replaces the staged inputs
        with pytest.raises(IdbError) as e:
            b.run()
        assert e.value.status == 8
        b.plan()
        b.run()
        clone, core, copies = b.results()
        o = oracle.cluster(w)
        assert np.array_equal(clone, o.clone_id) and np.array_equal(copies, o.copies)


def test_replay_learned_schedule_after_batch_plan():
    """The bench's sequence: a batch plan with the learned schedule on a
    context, then repeated host calls on the same context (eager, capture,
    replays), every one the oracle's answer."""
    from immunodbscan_gb300 import learned
    w = synth.workload(2, scale=0.01)
    o = oracle.cluster(w)
    with Context(0) as ctx:
        X, T = learned.profile(w, ctx)
        p, _ = learned.train(X, T, ctx, epochs=50)
        learned.install(ctx, p)
        b = DeviceBatch(w, ctx, schedule=1)
        b.plan()
        b.run()
        _same_triple(b.results(), o, "batch")
        for k in range(5):
            g = cluster_workload(w, ctx, schedule=1)
            _same(g, o, f"host call {k} (launches {g.stats.kernel_launches})")
        for k in range(3):
            g = cluster_workload(w, ctx, schedule=0)
            _same(g, o, f"static host call {k} (launches {g.stats.kernel_launches})")


def _same_triple(res, o, label):
    clone, core, copies = res
    assert np.array_equal(copies, o.copies), label
    assert np.array_equal(core, o.core), label
    assert np.array_equal(clone, o.clone_id), label
