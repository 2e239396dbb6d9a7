"""The bench's multi-rank plumbing on CPU: two gloo ranks (127.0.0.1) set
up from the launcher's environment, meet at the barrier and agree on the
maximum of their timings, which is what the N-GPU bench line divides the
whole job's work by."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), BFG_BENCH_GLOO="1")
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, dist = bench.dist_setup()
    try:
        bench.barrier(dist)
        m = bench.max_over_ranks(1.5 * (rank + 1), dist)
        q.put((r, w, local, m))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 2, 0, 3.0), (1, 2, 1, 3.0)]


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    env = {k: os.environ.pop(k) for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK") if k in os.environ}
    try:
        assert bench.dist_setup() == (1, 0, 0, None)
        assert bench.max_over_ranks(2.5, None) == 2.5
    finally:
        os.environ.update(env)
