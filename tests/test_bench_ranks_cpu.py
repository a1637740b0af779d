"""The bench's multi-GPU arithmetic (replicas: one heap per rank, no collective
on the data path) with two gloo ranks on CPU: the job's time is the slowest
rank's, its throughput every rank's pairs over that time."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    slowest = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
    q.put((rank, slowest, bench.job_throughput(1000, world, slowest)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]
    assert all(o[2] == pytest.approx(1000 * 2 / 15e-3) for o in out)


def test_single_rank_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.job_throughput(31129600, 1, 7.66) == pytest.approx(31129600 / 7.66e-3)
