"""The N > 1 host path of bench.py on CPU (gloo, world size 2, 127.0.0.1): the time reported is
the maximum over ranks, every rank passes the barriers, and under the reference arm only rank 0
works and prints while the other ranks exit 0 without output.  No GPU is used."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

torch = pytest.importorskip("torch")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


CHILD = r"""
import json, os, sys
sys.path.insert(0, {root!r})
import bench
world, rank, local, dist = bench.dist_setup()
bench.barrier(dist)
t = bench.max_over_ranks(dist, 1.5 + rank)
bench.barrier(dist)
print(json.dumps({{"world": world, "rank": rank, "max": t}}))
"""


def run_ranks(cmd, world=2, timeout=120):
    port = free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen(cmd, env=env, cwd=ROOT, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            o, e = p.communicate(timeout=timeout)
        except subprocess.TimeoutExpired:
            p.kill()
            o, e = p.communicate()
        outs.append((p.returncode, o, e))
    return outs


def test_max_over_ranks_and_barriers_gloo():
    outs = run_ranks([sys.executable, "-c", CHILD.format(root=ROOT)])
    for rc, o, e in outs:
        assert rc == 0, e
    res = [json.loads(o.strip().splitlines()[-1]) for _, o, _ in outs]
    assert sorted(r["rank"] for r in res) == [0, 1]
    assert all(r["world"] == 2 and r["max"] == 2.5 for r in res)


def test_reference_arm_runs_on_rank_zero_only():
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--size", "16",
           "--steps", "4", "--warmup", "2"]
    outs = run_ranks(cmd, timeout=300)
    (rc0, o0, e0), (rc1, o1, e1) = outs
    assert rc0 == 0 and rc1 == 0, (e0, e1)
    line = json.loads(o0.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == 2
    assert line["steps"] == 4 and line["warmup"] == 2   # the steps asked for, timed in full
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    assert o1.strip() == ""
