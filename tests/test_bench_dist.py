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


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` runs the CPU restatement of the path (no GPU needed) and prints
    one JSON line with the metric, the reference marker, its CPU baseline and an e2e without
    host-device copies."""
    import json
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True,
                       timeout=300, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "Mray-Gaussian evals/s"
    assert d["unit"] == "Mevals/s" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "Mevals/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
