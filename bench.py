"""Throughput of the DBSCAN clone-collapsing path on GB300.

Default workload: 64 synthetic amino-acid repertoires of log-uniform size
5k-500k (5.0M sequences), Hamming eps=1, minPts=2 -- the batched workload the
throughput target is quoted on.  A step clusters all 64 repertoires; with
Hamming eps <= 2 the library takes its candidate pairs from the segment join
(`candidates` in the JSON line), which scores fewer pairs than the admissible
count in the numerator.

Metric: Gpair-distances/s = admissible unique pairs (V and J overlap, admissible
length gap, counted once; a property of the workload, not of the schedule) per
second of device time; sequences/s alongside.

  value   batched path: one CUDA-graph replay per step (idb_batch_run) with the
          inputs resident in HBM; device time from CUDA events on the library's
          stream.  Inputs (~0.7 GB) and working set exceed the 129 MB L2.
  e2e     idb_cluster (the InterlinkClass replacement) with pinned host buffers:
          H2D of the columns, the whole path, D2H of clone_id/core/copies.
  plain   the same workload as 64 per-repertoire idb_cluster_device calls.

  parity  every row of the batched result against the oracle (indexed mode:
          the all-pairs answer); a mismatch ends the run with exit status 3.

`--impl reference` times the CPU restatement of the reference path (the
all-pairs oracle, OpenMP on all host cores) on a fixed sample of the same
workload (the smallest repertoires up to a row-pair budget), the rows the GPU
arm's cpu_baseline also clusters on the GPU; the reference's CUDA code has no
CPU backend.
"""
from __future__ import annotations

import argparse
import ctypes as C
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# More hardware work queues than CUDA's default 8, set before CUDA starts in
# this process: with torch's streams and several library contexts (three
# streams each) a shared queue serialised unrelated streams and stalled single
# idb_cluster calls by 20-30 ms.  A value set by the caller wins.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = ("Gpair-distances/s and sequences clustered/s, batched+learned vs plain "
          "(identical partitions)")
UNIT = "Gpair-distances/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", type=int, default=2)
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--mlp-epochs", type=int, default=200)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--tile", default=None,
                    help="work-unit shape RX,TY (x-entries per lane, y-chunk); skips the autotuner")
    ap.add_argument("--no-learned-w3", action="store_true",
                    help="skip the learned-versus-static comparison on the learned-scheduling "
                         "workload (workload 3, 500k rows)")
    ap.add_argument("--static-only", action="store_true",
                    help="time the static schedule only (no network is trained)")
    ap.add_argument("--candidates", default="auto", choices=["auto", "buckets"],
                    help="candidate pairs: automatic (the segment join for Hamming eps <= 2) or "
                         "every admissible pair of the buckets")
    ap.add_argument("--no-workloads", action="store_true",
                    help="skip the table of the other workloads (0, 1, 3 at 2M rows, 4 at 10M "
                         "rows: batched and plain device time, identical partitions)")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the check of every row against the oracle's indexed mode")
    ap.add_argument("--row-chunks", type=int, default=0,
                    help="e2e: row chunks the host columns are copied in (0 automatic)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# The CPU sample: the oracle in its all-pairs, full-DP mode (the reference's
# structure) visits n(n-1)/2 row pairs per repertoire, so the sample is the
# smallest repertoires up to a budget of row pairs -- the same rows in both
# arms.  A single repertoire above the budget is cut to its first rows.
CPU_SAMPLE_ROW_PAIRS = {True: 5e10, False: 5e8}   # Hamming / Levenshtein


def cpu_sample(w):
    """(repertoire ids, rows kept of the last one or None) of the CPU sample."""
    budget = CPU_SAMPLE_ROW_PAIRS[bool(w.use_hamming)]
    sizes = np.diff(w.rep_off).astype(np.float64)
    order = np.argsort(sizes, kind="stable")
    pick, acc = [], 0.0
    for r in order:
        c = sizes[r] * (sizes[r] - 1) / 2
        if pick and acc + c > budget:
            break
        pick.append(int(r))
        acc += c
    cut = None
    if len(pick) == 1 and acc > budget:
        cut = int(math.sqrt(2 * budget))
    return sorted(pick), cut


def sample_workload(w, pick, cut):
    from immunodbscan_gb300 import synth
    if cut is None:
        return w.subset_repertoires(pick)
    lo = int(w.rep_off[pick[0]])
    return synth.take_rows(w, np.arange(lo, lo + cut))


def run_cpu(w, threads: int):
    """The oracle (all-pairs, full DP) on the CPU sample; returns its rate and
    its answer."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    pick, cut = cpu_sample(w)
    sub = sample_workload(w, pick, cut)
    t0 = time.perf_counter()
    r = oracle.cluster(sub, n_threads=threads, max_candidates=0)
    dt = time.perf_counter() - t0
    return dict(value=r.admissible_pairs / dt / 1e9, seq_per_s=sub.n / dt, seconds=dt,
                rows=sub.n, reps=len(pick), pairs=r.admissible_pairs, pick=pick, cut=cut,
                result=r, sub=sub)


def sample_text(res):
    what = (f"first {res['cut']} rows of the workload" if res["cut"] is not None else
            f"{res['reps']} smallest repertoires of the workload")
    return f"{what} ({res['rows']} rows, {res['pairs']} admissible pairs)"


def full_parity(w, clone, core, copies, threads: int):
    """Every row of the timed workload against the oracle's indexed mode (pairs
    within the largest admissible length gap, edit distance cut off at eps:
    the all-pairs answer, tested in tests/test_oracle.py)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    t0 = time.perf_counter()
    o = oracle.cluster(w, n_threads=threads, max_candidates=0, indexed=True)
    dt = time.perf_counter() - t0
    bad = ((clone != o.clone_id) | (core != o.core) | (copies != o.copies))
    return {"rows": int(w.n), "repertoires": int(w.n_rep),
            "identical": bool(not bad.any()), "differing_rows": int(bad.sum()),
            "oracle": "oracle/oracle.cpp indexed mode (the all-pairs answer), "
                      f"{threads} host threads, {dt:.1f} s",
            "compared": "clone_id, core, copies of every row (batched path)",
            "n_clusters": int(o.n_clusters), "neighbour_pairs": int(o.neighbour_pairs)}


def profiled_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` on `workload` from the committed ncu
    summary (a line 'traffic_bytes_per_launch <kernel> <workload> <bytes>'), or
    None when no capture of that pair is committed."""
    d = os.path.join(ROOT, "profiles")
    try:
        names = sorted(os.listdir(d))
    except OSError:
        return None
    for nm in names:
        try:
            with open(os.path.join(d, nm)) as f:
                for line in f:
                    p = line.split()
                    if len(p) == 4 and p[0] == "traffic_bytes_per_launch" and p[1] == kernel \
                            and p[2] == workload:
                        return int(p[3])
        except OSError:
            continue
    return None


def measured_hbm_peak() -> float:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0


def workload_name(w):
    eps = (f"eps={w.abs_eps}" if w.threshold != w.threshold else
           f"threshold={w.threshold:g}" + (f" capped at {w.abs_eps}" if w.abs_eps >= 0 else ""))
    return (f"{w.name}: {w.n_rep} repertoire(s), {w.n} rows, "
            f"{'Hamming' if w.use_hamming else 'Levenshtein'} {eps}, minPts={w.min_pts}")


def reference_arm(args, world, rank, w):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    vals, secs = [], []
    for k in range(args.warmup + args.steps):
        res = run_cpu(w, threads)
        if k >= args.warmup:
            vals.append(res["value"])
            secs.append(res["seconds"])
    value = float(np.median(vals))
    sample = sample_text(res) + " per step, the same rows as the GPU arm's cpu_baseline"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(secs)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded generator)",
        "config": {"workload": workload_name(w), "global_batch": w.n * world,
                   "seq_len": int(w.lengths().max()),
                   "parallelism": f"host CPU, {threads} threads (rank 0)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def prediction_quality(w, ctx, shape, params):
    """How well the trained network predicts the work of the timed workload's
    bin pairs (a profile of that workload, not seen in training), next to the
    best the static cost can do: a least-squares line from log2(pairs) to the
    same measured log2 cycles."""
    from immunodbscan_gb300 import learned
    X, T = learned.profile(w, ctx, tune=shape)
    T = T.astype(np.float64)
    pred = learned.forward(params, X)
    f = X[:, 6].astype(np.float64)                 # log2(1 + pairs)
    A = np.stack([f, np.ones_like(f)], 1)
    coef = np.linalg.lstsq(A, T, rcond=None)[0]
    var = float(np.var(T)) or 1.0
    mse_mlp = float(np.mean((pred - T) ** 2))
    mse_static = float(np.mean((A @ coef - T) ** 2))
    return {"eval_binpairs": int(len(T)), "eval_mse_log2_cycles": mse_mlp,
            "eval_r2": 1.0 - mse_mlp / var, "static_fit_mse_log2_cycles": mse_static,
            "static_fit_r2": 1.0 - mse_static / var}


def time_batch(batch, steps, warmup, world, clocks=None):
    """Warm up, then time exactly `steps` graph replays (device time per step)."""
    import torch
    for _ in range(warmup):
        batch.run()
    if clocks:
        clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    ms, ms_dist, phases, launches = [], [], [], 0
    wall0 = time.perf_counter()
    for _ in range(steps):
        st = batch.run()
        ms.append(st.ms_total)
        ms_dist.append(st.ms_distance)
        phases.append([st.ms_phase[k] for k in range(5)])
        launches += st.kernel_launches
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    barrier(world)
    clk = clocks.stop() if clocks else None
    return dict(step_ms=allreduce_max(world, float(np.mean(ms))), ms_dist=float(np.mean(ms_dist)),
                phases=phases, launches=launches, wall=wall, last=st, clocks=clk)


def main():
    args = parse()
    world, rank, local = dist_init(args)
    from immunodbscan_gb300 import synth
    t0 = time.time()
    w = synth.workload(args.workload, scale=args.scale)
    w.candidates = 1 if args.candidates == "buckets" else 0
    gen_s = time.time() - t0
    if args.impl == "reference":
        reference_arm(args, world, rank, w)
        return
    import torch
    from immunodbscan_gb300 import Context, DeviceBatch, _lib, learned, tuning
    from immunodbscan_gb300.interlink import make_params
    torch.cuda.set_device(local)
    L = _lib.lib()
    # one context per captured plan: eager calls on a context may regrow its
    # workspace, which would invalidate a graph captured on it
    ctx_setup, ctx_static, ctx_learned = Context(local), Context(local), Context(local)
    n = w.n

    # numerator: admissible unique pairs (setup, untimed)
    inp, keep = build_host_input(w, pinned=False)
    prm0 = make_params(w.threshold, w.abs_eps, w.min_pts, w.use_hamming,
                       candidates=w.candidates)
    adm = C.c_uint64()
    _lib.check(L.idb_count_admissible(ctx_setup.handle, C.byref(inp), C.byref(prm0), C.byref(adm)))
    admissible = int(adm.value)

    # autotuner: work-unit shape measured on this workload (setup, untimed)
    if args.tile:
        shape = tuple(int(x) for x in args.tile.split(","))
        tune_rec = {"tried": [], "source": "--tile"}
    else:
        tune_rec = tuning.measure(w, ctx_setup)
        shape = (tune_rec["rx"], tune_rec["ty"])

    # learned schedule: trained on a profile of a differently seeded workload of
    # the same kind (setup, untimed)
    t0 = time.time()
    learn = not args.static_only
    X = T = None
    loss = float("nan")
    if learn:
        wt = synth.workload(args.workload, scale=min(args.scale, 0.1), seed=4242 + args.workload)
        wt.candidates = w.candidates
        X, T = learned.profile(wt, ctx_setup, tune=shape)
        params, loss = learned.train(X, T, ctx_setup, epochs=args.mlp_epochs)
        learned.install(ctx_learned, params)
    train_s = time.time() - t0

    # batched graph path, static heavy-first order
    b_static = DeviceBatch(w, ctx_static, schedule=0, tune=shape)
    b_static.plan()
    clocks = ClockSampler(local)
    r_static = time_batch(b_static, args.steps, args.warmup, world, None if learn else clocks)
    if learn:
        # batched graph path, learned order (the headline value)
        b_learned = DeviceBatch(w, ctx_learned, schedule=1, tune=shape)
        b_learned.plan()
        r = time_batch(b_learned, args.steps, args.warmup, world, clocks)
    else:
        b_learned, r = b_static, r_static
    step_ms = r["step_ms"]
    value = world * admissible / (step_ms * 1e-3) / 1e9
    last = r["last"]
    clone_b, core_b, copies_b = b_learned.results()
    clone_s, core_s, _ = b_static.results()

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u8",
           "data": "synthetic (seeded generator, no public dataset)",
           "config": {"workload": workload_name(w),
                      "global_batch": n * world, "seq_len": int(w.lengths().max()),
                      "parallelism": "replicas only" if world > 1 else "single GPU",
                      "l2": "inputs and working set larger than L2 (129 MB)",
                      "schedule": ("learned (2x64 MLP, BF16 inference)" if learn else
                                   "static (heavy-first by pair count)"),
                      "tile": {"rx": shape[0], "ty": shape[1], "source": "autotuner"}},
           "seq_per_s": world * n / (step_ms * 1e-3), "admissible_pairs": admissible,
           "candidates": "segment join" if last.candidates == 1 else "buckets (every admissible pair)",
           "pairs_evaluated": int(last.pairs_evaluated),
           "neighbour_pairs": int(last.neighbour_pairs), "n_uniques": int(last.n_uniques),
           "n_clusters": int(last.n_clusters), "gpu_launches": int(r["launches"]),
           "phase_ms": {k: float(np.mean([p[i] for p in r["phases"]])) for i, k in
                        enumerate(["front_dedupe", "buckets_schedule", "distance", "graph",
                                   "outputs"])},
           "ms_outside_phases": step_ms - float(np.mean([sum(p) for p in r["phases"]])),
           "wall_ms_per_step": 1e3 * r["wall"] / args.steps, "gen_seconds": gen_s,
           "clocks": r["clocks"],
           "static_schedule": {"ms_per_step": r_static["step_ms"],
                               "distance_ms": r_static["ms_dist"],
                               "learned_gain": r_static["step_ms"] / step_ms,
                               "pairs_evaluated": int(r_static["last"].pairs_evaluated),
                               "neighbour_pairs": int(r_static["last"].neighbour_pairs),
                               "n_clusters": int(r_static["last"].n_clusters),
                               "identical_partitions": bool(np.array_equal(clone_s, clone_b) and
                                                            np.array_equal(core_s, core_b)),
                               "differing_rows": int(np.count_nonzero((clone_s != clone_b) |
                                                                      (core_s != core_b)))},
           "autotune": {"tried": tune_rec["tried"]}}
    if learn:
        out["learned_model"] = {"train_binpairs": int(len(T)), "train_mse_log2_cycles": loss,
                                "setup_seconds": train_s, **prediction_quality(w, ctx_setup, shape,
                                                                                params)}
    else:
        out["config"]["tile"]["source"] = tune_rec.get("source", "autotuner")
        del out["static_schedule"]

    # roofline of the distance kernel: integer logic against the measured int peak
    gops = C.c_double()
    pms = C.c_double()
    L.idb_diag_int_peak(local, C.byref(gops), C.byref(pms))
    ops_pair = ops_per_pair(w, None)
    t_dist = r["ms_dist"] * 1e-3
    if w.use_hamming:
        work_ops = ops_pair * last.pairs_evaluated
    else:                       # Myers/Hyyro: ops per text column actually consumed
        work_ops = ops_pair * last.lev_columns
    achieved = work_ops / t_dist / 1e9 if t_dist > 0 else 0.0
    out["roofline"] = {"bound": "int", "achieved": achieved, "peak": gops.value,
                       "unit": "Gop/s (32-bit integer logic)",
                       "frac": achieved / gops.value if gops.value else None,
                       "traffic": (profiled_traffic("k_hamming", w.name)
                                   if w.use_hamming and args.scale == 1.0 else None),
                       "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                         "launch at scale 0.2, scaled by the rows to full size "
                                         "(profiles/k_hamming_workload2_scale0.2.md)",
                       "kernel": "k_hamming" if w.use_hamming else "k_levenshtein",
                       "ops_per_unit": ops_pair,
                       "work_unit": "pair" if w.use_hamming else "pair-column (text residue)",
                       "work_units": int(last.pairs_evaluated if w.use_hamming else last.lev_columns),
                       "kernel_ms": t_dist * 1e3,
                       "hit_fraction": (float(last.neighbour_pairs) / float(last.pairs_evaluated)
                                        if w.use_hamming and last.pairs_evaluated else None),
                       "peak_source": "measured: idb_diag_int_peak (lop3/add chains, all SMs)"}

    # graph / union-find / border / renumber phases against HBM bandwidth.  The
    # algorithmic bytes, kernel by kernel: init (copies read, count / parent /
    # border-minimum written: 16 n_u); count pass (edge 8 B, both ends' copies
    # 8 B, both ends' count updates 8 B: 24 E); core flags (8 n_u); union pass
    # (edge 8 B, both ends' core flags 8 B: 16 E, and both ends' parents for a
    # core-core edge: 8 E_cc); compress (12 n_u); scan of the root flags
    # (8 n_u); labels (core, parent, border minimum, rank, repertoire, first
    # unique read, label written: 28 n_u).  Border-minimum updates are left out.
    n_u, E, E_cc = int(last.n_uniques), int(last.neighbour_pairs), int(last.core_edges)
    graph_bytes = 40 * E + 8 * E_cc + 72 * n_u
    graph_ms = float(np.mean([p[3] for p in r["phases"]]))
    hbm_peak = measured_hbm_peak()
    out["roofline_graph"] = {"bound": "hbm", "achieved": graph_bytes / (graph_ms * 1e-3) / 1e9,
                             "peak": hbm_peak, "unit": "GB/s",
                             "frac": graph_bytes / (graph_ms * 1e-3) / 1e9 / hbm_peak,
                             "traffic": None, "phase_ms": graph_ms, "bytes": graph_bytes,
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}
    # the reference's own work on the same data: every unique pair of a table, plus
    # the second sweep over cores x uniques (each repertoire is one table there)
    rep_id = np.searchsorted(w.rep_off, np.arange(n), side="right") - 1
    is_rep = copies_b > 0
    nu_r = np.bincount(rep_id[is_rep], minlength=w.n_rep).astype(np.float64)
    nc_r = np.bincount(rep_id[is_rep & (core_b > 0)], minlength=w.n_rep).astype(np.float64)
    ref_pairs = float(np.sum(nu_r * (nu_r - 1) / 2 + nc_r * nu_r))
    out["reference_equivalent"] = {
        "pairs": ref_pairs, "unit": "Gpair-distances/s",
        "value": world * ref_pairs / (step_ms * 1e-3) / 1e9,
        "definition": "sum over repertoires of n_u(n_u-1)/2 + n_cores*n_u (the reference's "
                      "all-pairs core sweep plus its core x unique growth sweep)"}

    # e2e through idb_cluster (the InterlinkClass replacement) with pinned host buffers
    if not args.no_e2e:
        hin, hkeep = build_host_input(w, pinned=True)
        prm = make_params(w.threshold, w.abs_eps, w.min_pts, w.use_hamming, False, int(learn), shape,
                          w.candidates, row_chunks=args.row_chunks)
        clone = torch.empty(n, dtype=torch.int32).pin_memory()
        core = torch.empty(n, dtype=torch.int32).pin_memory()
        copies = torch.empty(n, dtype=torch.int32).pin_memory()
        est = _lib.Stats()
        o = _lib.Output(clone.data_ptr(), core.data_ptr(), copies.data_ptr(), None, None, None,
                        C.cast(C.pointer(est), C.c_void_p))
        # the first call runs eagerly, the second also captures the shape, the
        # rest replay it (idb_cluster's plan cache); a few replays before the
        # timed ones
        call_args = (ctx_learned.handle, C.byref(hin), C.byref(prm), C.byref(o))
        for _ in range(max(6, args.warmup)):
            _lib.check(L.idb_cluster(*call_args))
        barrier(world)
        times, dev_ms, dev_phases = [], [], []
        # the interpreter's cyclic garbage collector runs outside the timed
        # calls (a collection in this process can take tens of ms)
        gc.collect()
        gc.disable()
        try:
            for _ in range(args.steps):
                t0 = time.perf_counter()
                rc = L.idb_cluster(*call_args)
                times.append(time.perf_counter() - t0)
                _lib.check(rc)
                dev_ms.append(est.ms_total)
                dev_phases.append([est.ms_phase[k] for k in range(5)])
        finally:
            gc.enable()
        barrier(world)
        e2e_s = allreduce_max(world, float(np.mean(times)))
        h2d = sum(int(a.numel() * a.element_size()) for a in hkeep if isinstance(a, torch.Tensor))
        # breakdown: the same host->device copies alone; the span of the path on
        # the device (the call's own time stamps, from its first kernel to its
        # last: the columns arrive by row chunks during it, so it includes the
        # waits for the copies it overlaps); the result copies alone
        up_ms, down_ms = copy_times(hkeep, (clone, core, copies))
        out["e2e"] = {"value": world * admissible / e2e_s / 1e9, "unit": UNIT,
                      "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 12 * n,
                      "ms_per_step": e2e_s * 1e3, "seq_per_s": world * n / e2e_s,
                      "api": "idb_cluster (host buffers, %s schedule)" % ("learned" if learn else
                                                                           "static"),
                      "replayed": bool(est.kernel_launches > 0),
                      "ms_calls": [round(1e3 * t, 3) for t in times],
                      "ms_median": float(np.median(times)) * 1e3,
                      "breakdown_ms": {"upload_alone": up_ms, "device_span": float(np.mean(dev_ms)),
                                       "download_alone": down_ms,
                                       "batched_device_step": step_ms,
                                       "serial_sum": up_ms + step_ms + down_ms,
                                       "device_span_phases": dict(zip(
                                           ["front_dedupe (with the copies)", "buckets_schedule",
                                            "distance", "graph", "outputs"],
                                           np.mean(dev_phases, axis=0).tolist()))}}
        diff = ((clone.numpy().view(np.uint32) != clone_b) | (core.numpy() != core_b) |
                (copies.numpy().view(np.uint32) != copies_b))
        out["e2e"]["identical_partitions_vs_batched"] = bool(not diff.any())
        out["e2e"]["differing_rows"] = int(diff.sum())

    # plain per-repertoire path: one eager call per repertoire, default shape, static order
    if not args.no_plain:
        ctx_plain = Context(local)
        plain_ms = []
        subs = [DeviceBatch(w.subset_repertoires([rr]), ctx_plain) for rr in range(w.n_rep)]
        for sb in subs:
            sb.cluster_once()
        for _ in range(max(1, min(args.steps, 3))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for sb in subs:
                sb.cluster_once()
            torch.cuda.synchronize()
            plain_ms.append(1e3 * (time.perf_counter() - t0))
        pm = float(np.mean(plain_ms))
        same = True
        for rr, sb in enumerate(subs):
            c_, k_, p_ = sb.results()
            lo, hi = int(w.rep_off[rr]), int(w.rep_off[rr + 1])
            same &= np.array_equal(c_, clone_b[lo:hi]) and np.array_equal(k_, core_b[lo:hi])
        out["plain"] = {"value": admissible / (pm * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": pm,
                        "api": f"{w.n_rep} x idb_cluster_device (eager, per repertoire)",
                        "batched_learned_speedup": pm / step_ms,
                        "identical_partitions": bool(same)}
        ctx_plain.close()

    # the learned-scheduling workload: 2M-row-class repertoire with V/J usage
    # Zipf(1.8) (bin sizes 1 .. 10^5), Levenshtein eps=2; trained on a profile of
    # a differently seeded copy, timed against the static schedule
    if learn and not args.no_learned_w3 and args.workload == 2:
        out["learned_schedule_workload3"] = learned_vs_static(3, 1.0, 3, 2, world, local,
                                                              args.mlp_epochs)

    if rank == 0 and not args.no_workloads and args.workload == 2 and args.scale == 1.0:
        out["workloads"] = workload_table(local)
        out["csv_to_csv"] = csv_roundtrip()

    parity_ok = True
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        res = run_cpu(w, threads)
        # the GPU on the same rows, for a like-for-like rate
        sub = res["sub"]
        gb = DeviceBatch(sub, ctx_setup, schedule=0, tune=shape)
        gb.plan()
        rs = time_batch(gb, 5, 2, 1)
        cs_, ks_, ps_ = gb.results()
        o = res["result"]
        same = (np.array_equal(cs_, o.clone_id) and np.array_equal(ks_, o.core) and
                np.array_equal(ps_, o.copies))
        out["cpu_baseline"] = {"value": res["value"], "unit": UNIT, "cores": threads,
                               "kind": "port", "sample": sample_text(res) + f", {res['seconds']:.1f} s",
                               "gpu_same_sample": {"value": res["pairs"] / (rs["step_ms"] * 1e-3) / 1e9,
                                                   "ms_per_step": rs["step_ms"],
                                                   "identical_to_oracle": bool(same)}}
        parity_ok &= same
    if rank == 0 and not args.no_parity:
        out["parity"] = full_parity(w, clone_b, core_b, copies_b, os.cpu_count() or 1)
        parity_ok &= out["parity"]["identical"]
    if rank == 0:
        print(json.dumps(out), flush=True)
        if not parity_ok:
            sys.stderr.write("PARITY FAILURE: the GPU result differs from the oracle\n")
            sys.exit(3)
    for c in (ctx_setup, ctx_static, ctx_learned):
        c.close()


def workload_table(local, steps: int = 3, warmup: int = 2):
    """The other workloads at their full sizes: batched device time (a captured
    plan, static schedule, default tile) against one eager call of the plain
    path, with the partitions compared."""
    import torch
    from immunodbscan_gb300 import Context, DeviceBatch, _lib
    from immunodbscan_gb300.interlink import make_params
    L = _lib.lib()
    rows = []
    for k in (0, 1, 3, 4):
        t0 = time.time()
        w = synth_workload(k)
        gen = time.time() - t0
        ctx_b, ctx_p = Context(local), Context(local)
        try:
            inp, keep = build_host_input(w, pinned=False)
            prm = make_params(w.threshold, w.abs_eps, w.min_pts, w.use_hamming)
            adm = C.c_uint64()
            _lib.check(L.idb_count_admissible(ctx_p.handle, C.byref(inp), C.byref(prm), C.byref(adm)))
            b = DeviceBatch(w, ctx_b)
            b.plan()
            r = time_batch(b, steps, warmup, 1)
            clone_b, core_b, copies_b = b.results()
            st = r["last"]
            del b
            p = DeviceBatch(w, ctx_p)
            p.cluster_once()                       # warm
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            p.cluster_once()
            torch.cuda.synchronize()
            plain_ms = 1e3 * (time.perf_counter() - t1)
            clone_p, core_p, copies_p = p.results()
            del p
            same = (np.array_equal(clone_b, clone_p) and np.array_equal(core_b, core_p) and
                    np.array_equal(copies_b, copies_p))
            ms = r["step_ms"]
            rows.append({"workload": workload_name(w), "rows": int(w.n),
                         "admissible_pairs": int(adm.value), "ms_per_step": ms,
                         "seq_per_s": w.n / (ms * 1e-3),
                         "gpair_per_s": int(adm.value) / (ms * 1e-3) / 1e9,
                         "distance_ms": r["ms_dist"],
                         "phase_ms": {n: float(np.mean([ph[i] for ph in r["phases"]])) for i, n in
                                      enumerate(["front_dedupe", "buckets_schedule", "distance",
                                                 "graph", "outputs"])},
                         "plain_ms": plain_ms,
                         "plain_api": "idb_cluster_device (eager)",
                         "identical_partitions_plain_vs_batched": bool(same),
                         "candidates": "segment join" if st.candidates == 1 else "buckets",
                         "streamed": bool(st.streamed),
                         "neighbour_pairs": int(st.neighbour_pairs),
                         "n_clusters": int(st.n_clusters), "generate_s": gen})
        finally:
            ctx_b.close()
            ctx_p.close()
    return rows


_CSV_CONF = """input_settings
{
    separator "\\t"
    decimal "."
    endline "\\n"
    quotation "\\""
}
select_columns_to_read
{
    id_column_name "Sequence ID"
    v_gene_column_name "V-GENE and allele"
    j_gene_column_name "J-GENE and allele"
    cdr3_column_name "CDR3-IMGT"
}
gene_columns
{
    first_gene
    {
        name v_gene_column_name
        ref "@V@"
    }
    second_gene
    {
        name j_gene_column_name
        ref "@J@"
    }
}
sequence_columns
{
    name cdr3_column_name
}
maximum_absolute_edit_distance 1
minimum_number_of_neighbors 2
use_hamming true
output_prefix "output_"
output_suffix ""
output_filetype ".csv"
output_settings
{
    separator "\\t"
    decimal "."
    endline "\\n"
    quotation "\\0"
}
remove_noise_from_output false
select_columns_to_write
{
    id_column_name "ID.code"
    v_gene_column_name "V_CALL"
    cdr3_column_name "CDR3"
    cores "Cores"
    copies "Copies"
    clone_id "Clone"
}
benchmark_output_prefix "benchmark_"
benchmark_output_suffix ""
benchmark_output_filetype ".csv"
benchmark_output_settings
{
    separator "\\t"
    decimal "."
    endline "\\n"
    quotation "\\""
}
"""


def csv_roundtrip(scale: float = 0.2):
    """psdbscan (the command-line host) from a TSV file to a TSV file: the rows of
    20% of the bench workload (1.0M rows) as one table, Hamming eps=1.  Wall
    times of its reading, clustering and writing steps (its benchmark log)."""
    import shutil
    import tempfile
    from immunodbscan_gb300 import build, synth
    w = synth.workload(2, scale=scale)
    d = tempfile.mkdtemp(prefix="idb_csv_")
    try:
        vg, jg = os.path.join(d, "V.txt"), os.path.join(d, "J.txt")
        with open(vg, "wb") as f:
            f.write(b"\n".join(w.v_genes) + b"\n")
        with open(jg, "wb") as f:
            f.write(b"\n".join(w.j_genes) + b"\n")
        conf = os.path.join(d, "bench.conf")
        with open(conf, "w") as f:
            f.write(_CSV_CONF.replace("@V@", vg).replace("@J@", jg))
        inp = os.path.join(d, "rows.tsv")
        with open(inp, "wb") as f:
            f.write(b"Sequence ID\tV-GENE and allele\tJ-GENE and allele\tCDR3-IMGT\n")
            chunk = []
            for i in range(w.n):
                chunk.append(b"id%d\t%s\t%s\t%s\n" % (i, w.vcall(i), w.jcall(i), w.seq(i)))
                if len(chunk) == 100000:
                    f.write(b"".join(chunk))
                    chunk = []
            f.write(b"".join(chunk))
        t0 = time.perf_counter()
        r = subprocess.run([build.CLI, "--config_file", conf, "--input", inp], capture_output=True,
                           text=True, cwd=d)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            return {"error": (r.stdout + r.stderr)[-300:]}
        timers = {}
        with open(os.path.join(d, "benchmark_rows.csv")) as f:
            for line in f:
                p = line.rstrip("\n").split("\t")
                if len(p) == 2 and p[1].endswith(" sec"):
                    timers[p[0]] = float(p[1][:-4])
        return {"rows": int(w.n), "input_bytes": os.path.getsize(inp),
                "output_bytes": os.path.getsize(os.path.join(d, "output_rows.csv")),
                "read_s": timers.get("Reading Files"), "cluster_s": timers.get("Do clustering"),
                "write_s": timers.get("Writing Output"), "total_s": timers.get("Overall"),
                "wall_s": wall, "rows_per_s": w.n / wall,
                "api": "psdbscan --config_file --input (one table, Hamming eps=1, minPts=2)"}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def synth_workload(k):
    from immunodbscan_gb300 import synth
    return synth.workload(k)


def learned_vs_static(k, scale, steps, warmup, world, local, epochs):
    """Static and learned schedules on workload k at `scale` (the learned-
    scheduling workload: 2M rows, V/J usage Zipf(1.8), Levenshtein eps=2): the
    network is trained on bin-pair logs of runs of workloads 1 and 2 (the
    nucleotide Levenshtein and the batched amino-acid Hamming workloads), then
    the step times, the gain, the network's prediction error on this workload
    next to the static cost model's, and the equality of the partitions."""
    from immunodbscan_gb300 import Context, DeviceBatch, learned, synth, tuning
    w = synth.workload(k, scale=scale)
    ctx_s, ctx_l = Context(local), Context(local)
    try:
        rec = tuning.measure(w, ctx_s)
        shape = (rec["rx"], rec["ty"])
        Xs, Ts = [], []
        for kt, st in ((1, 0.25), (2, 0.1)):
            X, T = learned.profile(synth.workload(kt, scale=st), ctx_s)
            Xs.append(X)
            Ts.append(T)
        X, T = np.concatenate(Xs), np.concatenate(Ts)
        params, loss = learned.train(X, T, ctx_s, epochs=epochs)
        learned.install(ctx_l, params)
        bs = DeviceBatch(w, ctx_s, schedule=0, tune=shape)
        bs.plan()
        rs = time_batch(bs, steps, warmup, world)
        bl = DeviceBatch(w, ctx_l, schedule=1, tune=shape)
        bl.plan()
        rl = time_batch(bl, steps, warmup, world)
        cs, ks, _ = bs.results()
        cl, kl, _ = bl.results()
        q = prediction_quality(w, ctx_s, shape, params)
        return {"workload": workload_name(w), "tile": {"rx": shape[0], "ty": shape[1]},
                "trained_on": "bin-pair logs of workload 1 (25%) and workload 2 (10%)",
                "static_ms_per_step": rs["step_ms"], "learned_ms_per_step": rl["step_ms"],
                "static_distance_ms": rs["ms_dist"], "learned_distance_ms": rl["ms_dist"],
                "learned_gain": rs["step_ms"] / rl["step_ms"],
                "identical_partitions": bool(np.array_equal(cs, cl) and np.array_equal(ks, kl)),
                "train_binpairs": int(len(T)), "train_mse_log2_cycles": loss, **q}
    finally:
        ctx_s.close()
        ctx_l.close()


def copy_times(host_inputs, host_outputs, reps: int = 5):
    """Time (ms) of the host->device copies of the input columns and of the
    device->host copies of the outputs alone (pinned memory, CUDA events)."""
    import torch
    ins = [t for t in host_inputs if isinstance(t, torch.Tensor)]
    dev_in = [torch.empty_like(t, device="cuda") for t in ins]
    dev_out = [torch.empty_like(t, device="cuda") for t in host_outputs]
    host_out = [torch.empty_like(t).pin_memory() for t in host_outputs]   # leave the results
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(pairs):
        best = float("inf")
        for _ in range(reps):
            torch.cuda.synchronize()
            e0.record()
            for dst, src in pairs:
                dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best
    up = timed(list(zip(dev_in, ins)))
    down = timed(list(zip(host_out, dev_out)))
    del dev_in, dev_out, host_out
    return up, down


def ops_per_pair(w, batch) -> int:
    """Algorithmic 32-bit integer ops per evaluated pair of the distance kernel.

    Hamming (bit planes): one LOP3 per plane word folds XOR and OR, then the
    population test (eps==1: x & (x-1) == 0 -> 2 ops + 1 compare; otherwise
    popc + add per word + 1 compare).  Levenshtein: ops per text column per
    32-residue pattern word of the Myers/Hyyro step (Peq load, 4 LOP3, add,
    2 shifts/or, 2 LOP3 -> 16 with the code extraction).
    """
    L = int(w.lengths().max())
    Wd = max(1, (L + 31) // 32)
    planes = 2 if len(set(w.seq_blob.tolist()[:200000])) <= 4 else 5
    if w.use_hamming:
        if Wd == 1 and w.abs_eps == 1 and math.isnan(w.threshold):
            return planes + 3
        return planes * Wd + 2 * Wd + 1
    return 16 * Wd


def build_host_input(w, pinned: bool):
    """idb_input over host copies of the workload columns (pinned if asked)."""
    import torch
    from immunodbscan_gb300 import _lib
    from immunodbscan_gb300.interlink import _as_blob
    keep = []

    def host(a):
        t = torch.from_numpy(np.ascontiguousarray(a))
        if pinned:
            t = t.pin_memory()
        keep.append(t)
        return t.data_ptr()

    inp = _lib.Input()
    inp.n_rows = w.n
    inp.seqs, inp.seq_offsets = host(w.seq_blob if w.seq_blob.size else np.zeros(1, np.uint8)), host(w.seq_off)
    inp.v_calls, inp.v_offsets = host(w.v_blob), host(w.v_off)
    inp.j_calls, inp.j_offsets = host(w.j_blob), host(w.j_off)
    vb, vo = _as_blob(w.v_genes)
    jb, jo = _as_blob(w.j_genes)
    roff = np.ascontiguousarray(w.rep_off, np.uint32)
    keep += [vb, vo, jb, jo, roff]
    inp.v_genes, inp.v_gene_offsets, inp.n_v_genes = vb.ctypes.data, vo.ctypes.data, len(w.v_genes)
    inp.j_genes, inp.j_gene_offsets, inp.n_j_genes = jb.ctypes.data, jo.ctypes.data, len(w.j_genes)
    inp.n_repertoires = w.n_rep
    inp.rep_offsets = roff.ctypes.data
    return inp, keep


if __name__ == "__main__":
    main()
