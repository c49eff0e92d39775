"""The multi-GPU path of bench.py is replicas only (the step does not shard): each rank runs its
own cavity, the ranks meet at a barrier around the timed region, and rank 0 reports the sum of
cells x steps over the slowest rank's time. These tests run that host logic as two gloo ranks on
the CPU (127.0.0.1), and the reference arm under torchrun, where rank 0 alone runs and prints."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist(world, rank)
    d.barrier()
    slowest = d.max(10.0 * (rank + 1))  # this rank's "time"
    d.barrier()
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"max": slowest}, f)
    d.close()


def test_two_gloo_ranks_agree_on_the_slowest_time(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    pytest.importorskip("torch.distributed")
    port = free_port()
    mp.spawn(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    got = [json.load(open(tmp_path / f"r{k}.json"))["max"] for k in range(2)]
    assert got == [20.0, 20.0]


def test_reference_arm_under_torchrun_prints_once(orc, tmp_path):
    pytest.importorskip("torch.distributed")
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--grid", "48", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=tmp_path)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
