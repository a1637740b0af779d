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


def test_gpus_flag_starts_its_own_ranks():
    """`bench.py --gpus 2` without a launcher starts two ranks itself (under
    torch.distributed.run); in the reference arm rank 0 alone prints the one
    JSON line, with n_gpus 2 and the same config as the GB300 arm's."""
    import json
    import subprocess

    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--heap-gib", "0.0625", "--accessblock-mib", "8", "--ref-step-seconds", "0.2",
           "--rounds", "4"]
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_PORT")}
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["config"]["parallelism"] == "replicas"
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
    assert line["errors"] == {"nulls": 0, "pattern": 0}


def test_gpus_flag_must_match_the_launched_ranks():
    import subprocess

    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, timeout=120, env=env, cwd=ROOT)
    assert r.returncode != 0 and "--gpus 2 but 1 ranks were launched" in r.stderr
