"""Replicas-only multi-GPU accounting of bench.py, exercised with two gloo ranks on CPU: every rank runs its
own replica, the job's value is all ranks' operations over the slowest rank's time, and the reference arm
runs on rank 0 only."""

import io
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, results):
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = [2.0, 5.0][rank]  # rank 1 is the slow one
    value, worst = bench.replicas_value(1000, ms, ws, torch.device("cpu"))
    results[rank] = (value, worst)
    dist.barrier()
    dist.destroy_process_group()


def test_value_uses_the_slowest_rank():
    port = _free_port()
    with mp.Manager() as m:
        results = m.dict()
        mp.spawn(_rank, args=(2, port, results), nprocs=2, join=True)
        got = dict(results)
    for r in (0, 1):
        value, worst = got[r]
        assert worst == 5.0
        assert value == pytest.approx(2 * 1000 / 5e-3 / 1e6)


def test_single_rank_value():
    sys.path.insert(0, str(ROOT))
    import bench
    value, worst = bench.replicas_value(1000, 4.0, 1, torch.device("cpu"))
    assert worst == 4.0 and value == pytest.approx(1000 / 4e-3 / 1e6)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.reference_arm(bench.parse_args(["--impl", "reference", "--steps", "1", "--warmup", "0"]))
    assert buf.getvalue() == ""
