"""Learned schedule: the MLP's training kernel against a NumPy gradient, training
on profiled bin pairs, and identical partitions under the learned order.
The autotuner: every tried shape gives the same partition."""
import numpy as np
import pytest

from immunodbscan_gb300 import cluster_workload, learned, synth, tuning

pytestmark = pytest.mark.gpu


def test_mlp_gradient_matches_cpu(gpu_ctx):
    rng = np.random.default_rng(3)
    n = 777                                   # not a multiple of the 64-sample tile
    X = rng.normal(0, 1, size=(n, learned.F)).astype(np.float32)
    T = rng.normal(10, 3, size=n).astype(np.float32)
    p = learned.init_params(5)
    g_dev, loss_dev = learned.device_grad(p, X, T, gpu_ctx)
    g_cpu, loss_cpu = learned.cpu_grad(p, X, T)
    assert abs(loss_dev - loss_cpu) <= 1e-4 * max(1.0, loss_cpu)
    # FP32 accumulation in a different order than the float64 reference
    scale = np.abs(g_cpu).max()
    assert np.max(np.abs(g_dev - g_cpu)) <= 1e-4 * scale + 1e-5


def test_profile_train_and_learned_partitions(gpu_ctx):
    w = synth.workload(2, scale=0.01)
    X, T = learned.profile(w, gpu_ctx)
    assert len(T) > 100 and np.all(np.isfinite(X)) and np.all(T > 0)
    p0 = learned.init_params(0)
    loss0 = float(np.mean((learned.forward(p0, X) - T) ** 2))
    p, loss = learned.train(X, T, gpu_ctx, epochs=150)
    assert loss < 0.5 * loss0
    # the device forward agrees with the NumPy forward on the trained weights
    pred = learned.forward(p, X)
    assert np.corrcoef(pred, T)[0, 1] > 0.5
    base = cluster_workload(w, gpu_ctx)
    learned.install(gpu_ctx, p)
    try:
        got = cluster_workload(w, gpu_ctx, schedule=1)
    finally:
        learned.install(gpu_ctx, None)
    assert np.array_equal(got.clone_id, base.clone_id)
    assert np.array_equal(got.core, base.core)
    assert np.array_equal(got.copies, base.copies)


def test_network_predicts_better_than_static_cost(gpu_ctx):
    """What the trained network gains over the static schedule's cost model:
    on a profile of a workload it was not trained on, its error in log2 device
    cycles per bin pair is below that of the best straight line from log2(pairs)
    (fitted on that very profile, which favours the static model)."""
    wa = synth.workload(2, scale=0.03, seed=11)
    wb = synth.workload(2, scale=0.03, seed=12)
    Xa, Ta = learned.profile(wa, gpu_ctx)
    Xb, Tb = learned.profile(wb, gpu_ctx)
    p, _ = learned.train(Xa, Ta, gpu_ctx, epochs=300)
    mse_net = float(np.mean((learned.forward(p, Xb) - Tb) ** 2))
    A = np.stack([Xb[:, 6].astype(np.float64), np.ones(len(Tb))], 1)
    coef = np.linalg.lstsq(A, Tb.astype(np.float64), rcond=None)[0]
    mse_static = float(np.mean((A @ coef - Tb) ** 2))
    assert mse_net < mse_static, (mse_net, mse_static)


@pytest.mark.parametrize("k,scale", [(2, 0.004), (3, 0.004)])
def test_autotune_shapes_agree(gpu_ctx, tmp_path, k, scale):
    w = synth.workload(k, scale=scale)
    rec = tuning.measure(w, gpu_ctx)
    assert rec["tried"] and rec["ms"] > 0
    ref = cluster_workload(w, gpu_ctx)
    for t in rec["tried"][:4]:
        got = cluster_workload(w, gpu_ctx, tune=(t["rx"], t["ty"]))
        assert np.array_equal(got.clone_id, ref.clone_id)
    rx, ty, _ = tuning.shape_for(w, gpu_ctx, cache_path=str(tmp_path / "tune.json"))
    assert (rx, ty) == (rec["rx"], rec["ty"]) or rx > 0


def test_bf16_inference_matches_cpu_forward(gpu_ctx):
    """The scheduler's BF16 inference against two CPU forward passes on trained
    weights and profiled bin-pair features: a model of the same BF16 rounding
    (inputs, weights, hidden activations; only the summation order differs,
    FP32 on the device) within 1e-3 of the output range, and the exact float64
    network within the BF16 error budget (2% of the output range)."""
    w = synth.workload(2, scale=0.01)
    X, T = learned.profile(w, gpu_ctx)
    p, _ = learned.train(X, T, gpu_ctx, epochs=100)
    y_dev = learned.device_forward(p, X, gpu_ctx)
    y_bf16 = learned.forward_bf16(p, X)
    y_f64 = learned.forward(p, X)
    span = float(np.ptp(y_f64)) or 1.0
    assert np.max(np.abs(y_dev - y_bf16)) <= 1e-3 * span + 1e-3
    assert np.max(np.abs(y_dev - y_f64)) <= 2e-2 * span
    assert np.corrcoef(y_dev, y_f64)[0, 1] > 0.999


def test_autotune_picks_a_schedule_order():
    """With a model loaded the autotuner also times the learned order for the
    fastest shape and reports the faster order; both orders give the same
    partition."""
    from immunodbscan_gb300 import Context
    w = synth.workload(2, scale=0.01)
    with Context(0) as ctx:
        rec0 = tuning.measure(w, ctx)
        assert rec0["schedule"] == 0 and rec0["schedule_ms"][0] > 0 and rec0["schedule_ms"][1] == 0
        X, T = learned.profile(w, ctx)
        p, _ = learned.train(X, T, ctx, epochs=50)
        learned.install(ctx, p)
        rec = tuning.measure(w, ctx)
        assert rec["schedule"] in (0, 1)
        assert rec["schedule_ms"][0] > 0 and rec["schedule_ms"][1] > 0
        assert rec["schedule_ms"][rec["schedule"]] == min(rec["schedule_ms"])
        tune = (rec["rx"], rec["ty"])
        a = cluster_workload(w, ctx, schedule=0, tune=tune)
        b = cluster_workload(w, ctx, schedule=1, tune=tune)
        assert np.array_equal(a.clone_id, b.clone_id) and np.array_equal(a.core, b.core)
