"""The partition does not depend on the order in which the distance kernel takes
its work: eager calls, CUDA-graph replays under the static schedule and under
the learned schedule (with networks that give arbitrary orders), and several
work-unit shapes all give the oracle's clone ids, core flags and copies."""
import numpy as np
import pytest

import oracle
from immunodbscan_gb300 import Context, DeviceBatch, cluster_workload, learned, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batched_workload():
    w = synth.workload(2, scale=0.02)        # 64 repertoires, ~100k rows
    o = oracle.cluster(w)
    return w, o


def _same(got, o):
    clone, core, copies = got
    assert np.array_equal(core.astype(np.int32), o.core.astype(np.int32))
    assert np.array_equal(copies.astype(np.uint32), o.copies.astype(np.uint32))
    assert np.array_equal(clone.astype(np.uint32), o.clone_id.astype(np.uint32))


def test_eager_shapes_match_oracle(gpu_ctx, batched_workload):
    w, o = batched_workload
    for tune in [None, (4, 128), (8, 1024)]:
        r = cluster_workload(w, gpu_ctx, tune=tune)
        _same((r.clone_id, r.core, r.copies), o)


@pytest.mark.parametrize("model", ["static", "random", "scaled"])
def test_graph_replays_match_oracle(batched_workload, model):
    w, o = batched_workload
    ctx = Context(0)
    try:
        schedule = 0
        if model != "static":
            p = learned.init_params(11 if model == "random" else 12)
            if model == "scaled":
                p = p * 4.0               # large, spread predictions: many classes
            learned.install(ctx, p)
            schedule = 1
        b = DeviceBatch(w, ctx, schedule=schedule)
        b.plan()
        for _ in range(3):
            b.run()
            _same(b.results(), o)
    finally:
        ctx.close()
