"""The multi-rank bench logic on CPU with the gloo backend (world size 2): independent replicas,
whole-job throughput from the slowest rank, the reference arm run by rank 0 only."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]

WORKER = r"""
import os, sys, json
sys.path.insert(0, os.environ["ROOT"])
import numpy as np
import torch
import torch.distributed as dist
import bench
dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{os.environ['PORT']}",
                        rank=int(os.environ["RANK"]), world_size=2)
rank = dist.get_rank()
# rank r took 10 (r + 1) ms for 1000 units: the job took 20 ms for 2000 units
v, ms = bench.ranks_throughput(dist, 10.0 * (rank + 1), 1000, 2)
e, ems = bench.ranks_throughput(dist, 10.0 * (rank + 1), 1000, 2, reduce="min")
# per-rank replicas of the workload are seeded by rank (small sizes of the same generator)
from fluidlets_gb300.geometry import wall_sum_workload
T, S, F, eps = wall_sum_workload(64, 48, 16, 0.01, seed=rank)
digest = float(np.abs(T).sum() + np.abs(F).sum())
out = [None, None]
dist.all_gather_object(out, digest)
print(json.dumps({"rank": rank, "v": v, "ms": ms, "e": e, "ems": ems, "digests": out}), flush=True)
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_throughput_and_replicas():
    pytest.importorskip("torch.distributed")
    import json

    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, ROOT=str(ROOT), PORT=str(port), RANK=str(r), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e[-2000:]
        outs.append(json.loads(o.strip().splitlines()[-1]))
    for d in outs:
        assert d["ms"] == 20.0 and d["v"] == pytest.approx(2000 / 0.020)   # slowest rank's time
        assert d["e"] == pytest.approx(2000 / 0.020)                       # min over per-rank rates
        a, b = d["digests"]
        assert a != b                                                      # different replicas
    assert outs[0]["digests"] == outs[1]["digests"]


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    import bench

    class Args:
        warmup, steps, cpu_sample, gpus = 0, 1, 8, 2

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    bench.run_reference(Args())  # returns at once, prints nothing
    assert capsys.readouterr().out == ""
