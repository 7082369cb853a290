"""The multi-GPU path of bench.py is replicas only: each rank runs the whole
workload on its own GPU and the ranks meet only to time the step (a barrier
and a max over ranks).  That host logic is tested here with two gloo ranks
on the CPU, and the reference arm's rank behaviour with them."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import bench
d = bench.Dist()
d.barrier()
v = d.max(float(d.rank) + 0.5)
print(json.dumps({{"rank": d.rank, "world": d.world, "max": v}}), flush=True)
d.close()
"""


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


@pytest.fixture(scope="module")
def torch_dist():
    return pytest.importorskip("torch.distributed")


def run_ranks(code, world=2, timeout=120):
    port = free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=timeout)
        assert p.returncode == 0, e[-2000:]
        outs.append(o)
    return outs


def test_barrier_and_max_over_two_ranks(torch_dist):
    outs = run_ranks(RANK_SCRIPT.format(root=ROOT))
    got = sorted((json.loads(o.strip().splitlines()[-1]) for o in outs), key=lambda d: d["rank"])
    assert [g["rank"] for g in got] == [0, 1]
    assert all(g["world"] == 2 and g["max"] == 1.5 for g in got)


def test_reference_arm_prints_on_rank_zero_only(torch_dist, tmp_path):
    """bench.py --impl reference under two ranks: rank 0 prints one JSON line
    for the CPU port on a small cube, rank 1 exits 0 without output."""
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--n', '8', "
            "'--steps', '2', '--warmup', '1']; sys.path.insert(0, %r); import bench; bench.main()"
            % ROOT)
    outs = run_ranks(code, timeout=300)
    lines = [[l for l in o.splitlines() if l.startswith("{")] for o in outs]
    assert len(lines[0]) == 1 and lines[1] == []
    line = json.loads(lines[0][0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
