"""The N > 1 path of bench.py on the CPU (gloo, world size 2, 127.0.0.1).

The pass does not shard beyond replicas: every rank renders its own frame and
the only cross-rank steps are the barriers around the timed region, the max
of the ranks' times and the sum of their rays.  These run here over gloo:
the reductions of bench.Dist, and the reference arm launched as a multi-rank
job is launched (torchrun, two ranks: rank 0 prints one line, rank 1 exits
0 without work)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


RANK_SCRIPT = r"""
import os, sys
sys.path.insert(0, {root!r})
import bench
d = bench.Dist()
assert d.world == 2 and d.rank == int(os.environ["RANK"])
d.barrier()
assert d.max(float(d.rank) + 1.0) == 2.0
assert d.sum(float(d.rank) + 1.0) == 3.0
d.barrier()
d.close()
print("rank", d.rank, "ok")
"""


def test_dist_reductions_over_gloo():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            out, err = p.communicate(timeout=180)
        except subprocess.TimeoutExpired:
            p.kill()
            raise
        assert p.returncode == 0, err[-2000:]
        outs.append(out)
    assert "rank 0 ok" in outs[0] and "rank 1 ok" in outs[1]


def test_reference_arm_under_torchrun_two_ranks():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--width", "64", "--height", "36", "--grid", "32",
           "--spheres", "10", "--spp", "2", "--segments", "4", "--cpu-seconds", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
