"""The N > 1 path of bench.py on CPU: two gloo ranks (replicas) agree on the job's
time (the slowest rank's) and report the whole-job throughput."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    import torch
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = [10.0, 12.5][rank]  # rank 1 is the slow one
        torch.distributed.barrier()
        ms = bench.max_over_ranks(local_ms, "cpu")
        value = bench.job_value(1920 * 1080, 64, world, ms)
        q.put((rank, ms, value))
    finally:
        torch.distributed.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[1] for o in out] == [12.5, 12.5]
    expect = 1920 * 1080 * 64 * 2 / (12.5 / 1e3) / 1e6
    assert all(abs(o[2] - expect) < 1e-6 * expect for o in out)


def test_single_process_is_its_own_job():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(7.0, "cpu") == 7.0
    assert abs(bench.job_value(100, 10, 1, 1000.0) - 1e-3) < 1e-12
