"""CPU: the multi-process aggregation of bench.py (replicas, one per GPU) with
two gloo ranks: the job time is the slowest rank's, the pixel count the sum
over ranks, and the reference arm runs on rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import os, sys, json
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
rank = int(os.environ["RANK"]); world = int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo", rank=rank, world_size=world)
el, px = bench.aggregate(1.0 + rank, 100.0 * (rank + 1), world)
print(json.dumps({"rank": rank, "elapsed": el, "pixels": px}))
dist.destroy_process_group()
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _run_ranks(code, world, extra_args=()):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE=str(world), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", code, ROOT, *extra_args], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        outs.append(o)
    return outs


def test_aggregate_two_gloo_ranks():
    outs = _run_ranks(WORKER, 2)
    res = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    for r in res:
        assert r["elapsed"] == 2.0  # max over ranks
        assert r["pixels"] == 300.0  # sum over ranks


def test_aggregate_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.aggregate(1.5, 42.0, 1) == (1.5, 42.0)


REF_WORKER = r"""
import os, sys
sys.path.insert(0, sys.argv[1])
import bench
sys.argv = ["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-seconds", "0.1"]
bench.main()
"""


def test_reference_arm_prints_on_rank0_only(oracle):
    """Under two ranks only rank 0 runs the CPU reference arm and prints its line."""
    outs = _run_ranks(REF_WORKER, 2)
    lines0 = [l for l in outs[0].splitlines() if l.startswith("{")]
    lines1 = [l for l in outs[1].splitlines() if l.startswith("{")]
    assert len(lines0) == 1 and not lines1
    d = json.loads(lines0[0])
    assert d["impl"] == "reference" and d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["value"] > 0
