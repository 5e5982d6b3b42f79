"""The multi-process (replica) path of bench.py on CPU: torchrun with two
gloo ranks.  The reference arm runs on rank 0 alone and prints one JSON line;
the barrier and the max-over-ranks reduction the timed region uses agree on
every rank."""
import json
import os
import re
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def torchrun(args, timeout=300):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port())] + args
    env = dict(os.environ, OMP_NUM_THREADS="1")
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout, env=env)


def test_reference_arm_two_ranks():
    pytest.importorskip("torch")
    r = torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
                  "--workload", "icosphere_320", "--scaffold", "off"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1   # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0


SCRIPT = r'''
import os, sys
sys.path.insert(0, os.getcwd())
import bench
rank, world = bench.dist_setup(2)
bench.barrier(world)
m = bench.allreduce_max(float(rank + 1), world)
print("RANK%d %g %d" % (rank, m, world), flush=True)
import torch.distributed as dist
dist.destroy_process_group()
'''


def test_barrier_and_max_over_ranks(tmp_path):
    pytest.importorskip("torch")
    script = tmp_path / "dist_probe.py"
    script.write_text(SCRIPT)
    r = torchrun([str(script)])
    assert r.returncode == 0, r.stderr[-2000:]
    # the two ranks share stdout: their lines may arrive unseparated
    got = sorted(re.findall(r"RANK\d \S+ \d", r.stdout))
    assert got == ["RANK0 2 2", "RANK1 2 2"]
