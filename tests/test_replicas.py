"""Replica aggregation of bench.py under torch.distributed (world size 2, gloo on CPU): every
rank gets the slowest rank's time, and the value counts the voxel-steps of all ranks."""
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


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        ms, value = bench.replica_aggregate(1.0e9, 3, 100.0 + 50.0 * rank, world, "cpu")
        q.put((rank, ms, value))
    finally:
        dist.destroy_process_group()


def test_replica_aggregate_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in got:
        assert ms == 150.0
        assert value == pytest.approx(1.0e9 * 3 * 2 / 0.150)


def test_replica_aggregate_single_process():
    sys.path.insert(0, ROOT)
    import bench
    ms, value = bench.replica_aggregate(2.0e9, 4, 80.0, 1, "cpu")
    assert ms == 80.0 and value == pytest.approx(2.0e9 * 4 / 0.080)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Under torchrun the reference arm (CPU) runs on rank 0 alone; other ranks print nothing."""
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    bench.run_reference(argparse.Namespace(workload="tn", steps=1, warmup=0, cpu_seconds=0.1))
    assert capsys.readouterr().out == ""
