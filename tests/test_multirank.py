"""The multi-rank host path of bench.py on CPU: world_size 2 over gloo (127.0.0.1).

The solve path does not shard (each rank runs an independent replica), so the multi-rank
logic is the rendezvous, the barriers around the timed region, the max over ranks and
rank-0-only output; the reference arm runs on rank 0 alone and the other ranks exit 0."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


_WORKER = r"""
import os, sys
sys.path.insert(0, {root!r})
import bench
rank, world, local, pg = bench.dist()
assert world == 2 and pg is not None
bench.barrier(pg)
m = bench.allmax(pg, float(rank + 1) * 10.0)
print("RESULT", rank, m, flush=True)
bench.barrier(pg)
"""


def test_allmax_and_barrier_over_gloo():
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", _WORKER.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    got = sorted(line.split()[1:] for o, _ in outs for line in o.splitlines() if line.startswith("RESULT"))
    assert got == [["0", "20.0"], ["1", "20.0"]]


def test_reference_arm_under_torchrun_two_ranks():
    """`bench.py --impl reference` launched like the multi-GPU run: rank 0 prints one JSON line,
    rank 1 exits 0 without work."""
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--workload", "disks24"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == 2
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
