"""bench.py's multi-rank logic on two CPU ranks (gloo): the process group comes
up from the torchrun environment, the barrier passes, and every rank reports
the maximum of the ranks' step times.  The path runs as replicas only (one
process per GPU, no exchange on the data path), so this is all of its
multi-GPU host logic."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_init(None)
    bench.barrier(w)
    m = bench.allreduce_max(w, 1.5 + rank)
    q.put((r, w, local, m, dist.get_backend()))
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_max_step_time():
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=180) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert res == [(0, 2, 0, 2.5, "gloo"), (1, 2, 1, 2.5, "gloo")]
    assert all(p.exitcode == 0 for p in procs)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert bench.dist_init(None) == (1, 0, 0)
    assert bench.allreduce_max(1, 3.25) == 3.25
