"""bench.py's multi-rank plumbing on CPU (gloo, world size 2): the job time is the slowest
rank's, the value counts every rank's replica, and the reference arm runs on rank 0 only.
The GPU path runs one replica per GPU with no data-path collective (replicas only)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

_RANK = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
dist.init_process_group("gloo", init_method="tcp://127.0.0.1:{port}", rank={rank}, world_size=2)
mine = [120.0, 80.0][{rank}]
t = bench.max_over_ranks(mine, dist, "cpu")
print(json.dumps({{"rank": {rank}, "max": t, "value": bench.job_value(1000, 2, 4, t)}}))
dist.destroy_process_group()
"""


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_gloo():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = [subprocess.Popen([sys.executable, "-c", _RANK.format(root=str(ROOT), port=port, rank=r)],
                              stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["max"] == 120.0
        assert o["value"] == pytest.approx(1000 * 2 * 4 / 0.120)


def test_reference_arm_runs_on_rank_zero_only(capsys, monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup = 1, 3

    bench.run_reference(A())
    assert capsys.readouterr().out == ""
