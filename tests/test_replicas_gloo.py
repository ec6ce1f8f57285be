"""The N > 1 path of bench.py on the CPU: the solve does not shard, so N
ranks run N independent replicas, and the whole-job throughput is every
rank's work over the slowest rank's time (one all-reduce MAX).  Two gloo
ranks stand in for two GPUs."""
import json
import os
import socket
import subprocess
import sys

from conftest import ROOT

RANK_CODE = r"""
import json, os, sys
sys.path.insert(0, os.environ["REPO_ROOT"])
import torch.distributed as dist
dist.init_process_group("gloo")
import bench
rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
ms = [10.0, 25.0, 17.5, 4.0][rank]
value, max_ms = bench.replicas_throughput(ms, 1000, world)
print(json.dumps({"rank": rank, "value": value, "max_ms": max_ms}), flush=True)
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_ranks(world):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(r),
                   WORLD_SIZE=str(world), LOCAL_RANK=str(r), REPO_ROOT=ROOT, CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_CODE], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    out = []
    for p in procs:
        so, se = p.communicate(timeout=180)
        assert p.returncode == 0, se
        out.append(json.loads(so.strip().splitlines()[-1]))
    return sorted(out, key=lambda d: d["rank"])


def test_two_replicas_report_the_slowest_rank():
    res = _run_ranks(2)
    for d in res:
        assert d["max_ms"] == 25.0
        assert abs(d["value"] - 2 * 1000 / 0.025) < 1e-6


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    value, ms = bench.replicas_throughput(8.0, 500, 1)
    assert ms == 8.0 and abs(value - 500 / 0.008) < 1e-9
