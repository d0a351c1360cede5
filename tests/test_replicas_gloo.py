"""The multi-GPU path of bench.py is independent replicas (the k-truss sweep
does not shard); the host side that joins them - barrier, max of the timed
region over ranks, sum of the work - is exercised here with two gloo ranks
on the CPU."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import os, sys
sys.path.insert(0, {root!r})
import bench
d = bench.Dist()
d.barrier()
mx = d.max(float(d.rank + 1) * 10.0)
sm = d.sum(float(d.rank + 1))
assert (d.world, mx, sm) == (2, 20.0, 3.0), (d.world, mx, sm)
d.barrier()
d.close()
print("rank", d.rank, "ok")
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_gloo_join():
    pytest.importorskip("torch")
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", SCRIPT.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    outs = [p.communicate(timeout=240)[0] for p in procs]
    for p, o in zip(procs, outs):
        assert p.returncode == 0, o
        assert "ok" in o
