"""bench.py's replica path on CPU: two gloo ranks, the max over ranks of the step time, rank 0 alone printing,
the reference arm doing no work on ranks other than 0."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, os, sys
sys.path.insert(0, %r)
import bench
rank, world, local = bench.dist_setup()
t = bench.reduce_max(0.25 + rank, world)
s = bench.reduce_sum(rank + 1, world)
bench.barrier(world)
print(json.dumps({"rank": rank, "world": world, "max": t, "sum": s}))
"""


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_ranks(code, world=2, extra=()):
    port = _port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", code] + list(extra), env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True, cwd=ROOT))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(out)
    return outs


def test_max_and_sum_over_two_gloo_ranks():
    outs = _run_ranks(CHILD % ROOT)
    recs = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert sorted(r["rank"] for r in recs) == [0, 1]
    for r in recs:
        assert r["world"] == 2 and r["max"] == 1.25 and r["sum"] == 3.0


def test_reference_arm_runs_on_rank_zero_only():
    code = "import sys; sys.path.insert(0, %r); import bench; bench.run_reference(bench.parse())" % ROOT
    outs = _run_ranks(code, extra=["--impl", "reference", "--config", "c0", "--steps", "1", "--cpu-iters", "1"])
    line = json.loads(outs[0].strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert outs[1].strip() == ""            # rank 1 returned without work or output
