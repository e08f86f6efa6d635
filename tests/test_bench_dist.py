"""The replicas' aggregation of bench.py across ranks (world size 2, gloo on the CPU): every rank
reports the whole job's units over the slowest rank's time."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys

    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        value, dev_s = bench.job_value(0.5 + rank, 1e6, 10, world, torch.device("cpu"))
        out.put((rank, value, dev_s))
    finally:
        dist.destroy_process_group()


def test_job_value_takes_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for _, value, dev_s in res:
        assert dev_s == pytest.approx(1.5)
        assert value == pytest.approx(2 * 1e6 * 10 / 1.5 / 1e6)
