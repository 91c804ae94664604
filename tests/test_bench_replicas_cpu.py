"""bench.py's replica logic with two gloo processes on the CPU: the barrier
and the reduction that turns per-rank times and units into the whole-job
rate (the slowest rank's time, every rank's units)."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys, json
sys.path.insert(0, sys.argv[1])
import bench
rank, world, local = bench.dist_context()
bench.replica_barrier()
t, u = bench.reduce_replicas(1.0 + rank, 10 * (rank + 1))
print(json.dumps({"rank": rank, "world": world, "t": t, "u": u}))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reduce_time_and_units():
    pytest.importorskip("torch")
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(r), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    import json
    for (out, err), p in zip(outs, procs):
        assert p.returncode == 0, err
        d = json.loads(out.strip().splitlines()[-1])
        assert d["world"] == 2 and d["t"] == 2.0 and d["u"] == 30.0


def test_single_process_is_its_own_job():
    import bench
    assert bench.dist_context() == (0, 1, 0)
    assert bench.reduce_replicas(2.5, 7) == (2.5, 7.0)
