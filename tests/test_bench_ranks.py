"""The bench's multi-rank aggregation (replicas: barrier on both sides of the
timed region, max time over ranks, whole-job throughput) with two gloo ranks
on the CPU."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, lr = bench.dist_setup()
    bench.barrier(w)
    my_ms = 10.0 + 5.0 * r           # rank 1 is the slower replica
    got = bench.max_over_ranks(my_ms, w)
    bench.barrier(w)
    q.put((r, w, lr, got, bench.whole_job_tflops(5.41e9, got, w)))
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[3] == 15.0 for o in out)                 # every rank sees the slowest rank's time
    expected = 2 * 5.41e9 / 15e-3 / 1e12
    assert all(abs(o[4] - expected) < 1e-12 for o in out)


def test_single_rank_defaults():
    sys.path.insert(0, ROOT)
    import bench
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        assert bench.dist_setup() == (1, 0, 0)
        assert bench.max_over_ranks(3.0, 1) == 3.0
        assert bench.whole_job_tflops(1e12, 1000.0, 1) == pytest.approx(1.0)
    finally:
        os.environ.update(env)
