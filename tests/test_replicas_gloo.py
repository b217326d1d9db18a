"""The N>1 path of bench.py on CPU: world_size-2 gloo process groups.  Replicas share nothing
but the timing barrier and the max/sum reductions; the reference arm runs on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_WORKER = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import bench
world, rank, local, pg = bench.dist_setup(None)
bench.barrier(pg)
out = {"world": world, "rank": rank, "local": local,
       "max": bench.max_over_ranks(pg, 1.5 + rank), "sum": bench.sum_over_ranks(pg, 10.0 * (rank + 1))}
bench.barrier(pg)
print(json.dumps(out))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_timing_reductions():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", _WORKER, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    res = sorted((json.loads(o.strip().splitlines()[-1]) for o, _ in outs), key=lambda r: r["rank"])
    assert [r["rank"] for r in res] == [0, 1] and all(r["world"] == 2 for r in res)
    assert all(r["max"] == 2.5 for r in res)  # slowest replica's time
    assert all(r["sum"] == 30.0 for r in res)  # units processed by all replicas


def test_reference_arm_runs_on_rank_zero_only():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--workload", "convection_box", "--cpu-cores", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT,
                       env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
