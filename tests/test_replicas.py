"""bench.py's multi-rank path (replicas only) with two gloo ranks on the host:
the job time is the slowest rank's, the job throughput counts every rank's
units, and the reference arm runs on rank 0 alone."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_WORKER = r"""
import json, os, sys, time
sys.path.insert(0, sys.argv[1])
import torch, torch.distributed as dist
import bench
rank, world, _ = bench.env_rank()
dist.init_process_group("gloo")
out = {"rank": rank, "world": world}
out["max"] = bench.max_over_ranks(torch, dist, 1.5 + rank)       # per-rank "times"
out["value"] = bench.job_throughput(1000, world, out["max"])
class A:  # the reference arm's arguments; rank 1 must return without work
    gpus, steps, warmup, t10_n = world, 1, 0, 60
t0 = time.perf_counter()
if rank != 0:
    bench.run_reference(A)
out["reference_s"] = time.perf_counter() - t0
dist.barrier()
dist.destroy_process_group()
print(json.dumps(out), flush=True)
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", _WORKER, ROOT], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    import json
    outs = []
    for p in procs:
        so, se = p.communicate(timeout=240)
        assert p.returncode == 0, se[-2000:]
        outs.append(json.loads(so.strip().splitlines()[-1]))
    for o in outs:
        assert o["world"] == 2
        assert o["max"] == 2.5                 # the slower rank's time
        assert o["value"] == 2 * 1000 / 2.5    # units of both ranks over that time
    assert outs[1]["reference_s"] < 5.0        # rank 1 did no reference work
