"""The multi-process path of bench.py on CPU (gloo, world size 2): replicas only, the timing is the max
over ranks, and the reference arm runs on rank 0 alone."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        ws, r, local = bench._dist()
        assert (ws, r, local) == (world, rank, rank)
        # each rank times its own replica; the job's time is the slowest rank's
        t = bench._barrier_max(1.0 + rank, ws)
        out[rank] = t
    finally:
        dist.destroy_process_group()


def test_barrier_max_over_ranks():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        assert dict(out) == {0: 2.0, 1: 2.0}


def test_reference_arm_only_on_rank_zero(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class A:
        gpus, steps, warmup = 2, 1, 3

    assert bench.run_reference(A()) == 0
    assert capsys.readouterr().out == ""  # rank 1 prints nothing and does no work
