"""Replicas-only multi-GPU path of bench.py on CPU: two gloo ranks, each
with its own problem size and step times, reduce to the whole-job rate
(units of all ranks over the slowest rank's mean step time). No GPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env()[:2] == (rank, world)
        units = [1000.0, 3000.0][rank]
        times = [[0.5, 0.7], [0.9, 1.1]][rank]
        rate, step = bench.job_throughput(units, times, world)
        out.put((rank, rate, step))
    finally:
        dist.destroy_process_group()


def test_job_throughput_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    for _, rate, step in got:
        assert step == pytest.approx(1.0)          # slowest rank's mean step
        assert rate == pytest.approx(4000.0 / 1.0)  # all ranks' units over it


def test_job_throughput_single_rank():
    sys.path.insert(0, ROOT)
    import bench

    rate, step = bench.job_throughput(600.0, [0.2, 0.4], 1)
    assert step == pytest.approx(0.3) and rate == pytest.approx(2000.0)
