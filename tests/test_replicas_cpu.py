"""Replica (multi-rank) logic of bench.py on CPU: gloo, world size 2.

The path shards as independent replicas (one per GPU, no data exchange): the whole-job
throughput is the pairs of all ranks over the slowest rank's time, and the reference arm runs on
rank 0 alone.  These tests run the reductions through a real gloo process group.
"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    # rank r processed 100 (r + 1) pairs in 10 + r ms
    value, pairs, ms = bench.replica_throughput(100.0 * (rank + 1), 10.0 + rank, ws)
    bench.barrier(ws)
    out[rank] = (value, pairs, ms)
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    ws = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_worker, args=(ws, _free_port(), out), nprocs=ws, join=True)
    for r in range(ws):
        value, pairs, ms = out[r]
        assert pairs == 300.0
        assert ms == 11.0
        assert value == pytest.approx(300.0 / 0.011)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_throughput(500.0, 2.0, 1) == (250000.0, 500.0, 2.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    args = bench.parse(["--impl", "reference", "--gpus", "2"])
    assert bench.run_reference(args) == 0
    assert capsys.readouterr().out == ""


def test_reference_arm_json_line(monkeypatch, capsys):
    # the reference arm lists whole trajectory frames on the host cores: its JSON line carries
    # the contract's keys (one rank), and the GPU arm's metric and config
    import json
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.delenv("RANK", raising=False)
    args = bench.parse(["--impl", "reference", "--steps", "2", "--warmup", "1", "--n", "32768"])
    assert bench.run_reference(args) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "pairs/s" and line["value"] > 0
    assert line["steps"] == 2 and line["warmup"] == 1
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "pairs/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    L = (32768 / 0.85) ** (1.0 / 3.0)
    assert line["metric"] == bench.METRIC
    assert line["config"] == bench.workload_config(32768, L)
    assert line["ms_per_step"] > 0
    # every point of every frame is listed: about 8.8 ordered pairs per point at this density
    assert 8.0 * 32768 < line["pairs_per_step"] < 9.7 * 32768
