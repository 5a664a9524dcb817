"""The N > 1 host logic of bench.py on CPU: two gloo ranks stand in for two GPUs.  Replicas only
(each rank steps its own block): the barrier around the timed region, the maximum of the ranks'
times, the whole-job rate, and the reference arm's rank-0-only output."""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import bench
world, rank, local = bench.dist_init("gloo")
bench.barrier(world)
t = bench.max_over_ranks(0.5 + rank, world)           # rank 1 is the slower one
rate = bench.aggregate_rate(1000, 10, t, world)
import io, contextlib
buf = io.StringIO()
class A:                                              # the reference arm on a rank other than 0
    pass
if rank != 0:
    with contextlib.redirect_stdout(buf):
        bench.ref_arm(A(), world, rank)
bench.barrier(world)
print(json.dumps({"rank": rank, "world": world, "local": local, "t": t, "rate": rate, "ref_out": buf.getvalue()}))
import torch.distributed as dist
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replicas_gloo(tmp_path):
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD, REPO], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err[-3000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    by_rank = {o["rank"]: o for o in outs}
    assert set(by_rank) == {0, 1}
    for o in outs:
        assert o["world"] == 2
        assert o["t"] == 1.5                       # the slowest rank's time, on every rank
        assert o["rate"] == pytest.approx(2 * 1000 * 10 / 1.5)
    assert by_rank[1]["ref_out"] == ""             # only rank 0 runs and prints the reference arm


def test_single_process_needs_no_process_group(monkeypatch):
    sys.path.insert(0, REPO)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_init() == (1, 0, 0)
    assert bench.max_over_ranks(0.25, 1) == 0.25
    assert bench.aggregate_rate(64 ** 3, 10, 0.5, 1) == pytest.approx(64 ** 3 * 20)
