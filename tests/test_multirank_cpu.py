"""The bench's multi-replica logic on the CPU (gloo backend, world size 2).

Every box in this build has one GPU, so N > 1 runs one independent replica per rank: each
rank times its own steps, the job's time is the slowest rank's (an all-reduce MAX), and the
value is all ranks' operations over that time.  The collective and the aggregation run here
with gloo; the reference arm is launched through torch.distributed.run with two ranks, where
rank 0 alone times and prints and rank 1 exits without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


RANK_SCRIPT = r"""
import os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
dist.init_process_group("gloo", rank=int(os.environ["RANK"]), world_size=int(os.environ["WORLD_SIZE"]))
rank = dist.get_rank()
ms = bench.max_over_ranks(10.0 + 5.0 * rank, "cpu")
print("MAX", ms, "RATE", bench.job_rate(dist.get_world_size(), 1000, 4, ms))
dist.barrier()
dist.destroy_process_group()
"""


def test_max_over_ranks_and_job_rate_gloo():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=300) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err[-2000:]
        fields = out.split()
        assert fields[0] == "MAX" and float(fields[1]) == 15.0          # the slower rank's time
        assert float(fields[3]) == pytest.approx(2 * 1000 * 4 / 0.015)  # both ranks' ops / that time


def test_job_rate():
    assert bench.job_rate(1, 3 * 2 ** 20, 5, 1000.0) == pytest.approx(3 * 2 ** 20 * 5)
    assert bench.job_rate(4, 100, 2, 10.0) == pytest.approx(4 * 100 * 2 / 0.01)


def test_reference_arm_under_two_ranks():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--count", "256"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [line for line in r.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]                          # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
