"""The multi-GPU path of bench.py is replicas only: every rank solves its own copy and
the job's time is the slowest rank's.  Checked with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, loc = bench.dist_env()
        ms = 10.0 + 5.0 * rank                      # rank 1 is the slow replica
        job = bench.max_over_ranks(ms, w, torch.device("cpu"))
        out.put((r, w, loc, job, bench.replica_throughput(1000, job, w)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_replica():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[3] == 15.0 for r in res)           # both ranks report the max
    assert all(abs(r[4] - 2 * 1000 / 15e-3) < 1e-6 for r in res)


def test_single_rank_is_unchanged():
    import bench
    assert bench.max_over_ranks(12.5, 1, None) == 12.5
    assert bench.replica_throughput(100, 10.0, 1) == 100 / 10e-3
