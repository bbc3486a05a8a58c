"""bench.py host logic on CPU: the reference arm's JSON line, and the
multi-rank aggregation (max over ranks, rank-0-only output) over gloo with
two processes on 127.0.0.1."""
import json
import os
import socket
import subprocess
import sys

import pytest

from tests.conftest import ROOT


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "lj32k",
                        "--steps", "3", "--warmup", "3"], capture_output=True, text=True, timeout=300, check=True)
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "atom-steps/s" and d["unit"] == "atom-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["config"]["workload"] == "lj32k"


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


WORKER = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import bench
ws, rank, local = bench.dist_env()
dist = bench.init_pg(ws, False)
t = bench.reduce_max(dist, float(rank + 1))
bench.barrier(dist)
print(json.dumps({{"rank": rank, "max": t}}), flush=True)
if rank == 1:
    class A: pass
    a = A(); a.workload = "lj32k"; a.steps = 3; a.warmup = 3
    bench.run_reference_arm(a, ws, rank)   # non-zero ranks print nothing
dist.destroy_process_group()
"""


def test_two_rank_aggregation_gloo(tmp_path):
    script = tmp_path / "w.py"
    script.write_text(WORKER.format(root=ROOT))
    port = str(_free_port())
    procs = []
    for rank in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=port)
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    res = [json.loads([l for l in o.splitlines() if l.startswith("{")][0]) for o, _ in outs]
    assert all(r["max"] == 2.0 for r in res)
    # rank 1 ran the reference arm and printed no JSON line of its own
    assert sum(1 for l in outs[1][0].splitlines() if l.startswith("{")) == 1
