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


def test_reference_arm_line_on_rank_zero(monkeypatch, capsys):
    """Rank 0 prints the reference arm's one JSON line with the keys of the benchmark contract: full CPU CG
    solves by the oracle (one per step, no extrapolation), a cpu_baseline describing the run, an e2e equal
    to the value with no host-device bytes, and the same config string as the GPU arm for the system."""
    import json

    sys.path.insert(0, ROOT)
    import bench

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    monkeypatch.setattr(bench, "WORKLOAD", "lap2d_512")
    monkeypatch.setattr(bench, "TOL", 1e-8)

    class A:
        gpus, steps, warmup = 1, 1, 0

    assert bench.run_reference(A()) == 0
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "s" and d["higher_is_better"] is False
    assert d["value"] > 0 and abs(d["ms_per_step"] - 1e3 * d["value"]) < 1e-9
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["cores"] >= 1 and "lap2d_512" in d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # 939 iterations to 1e-8 on the 512^2 Laplacian, as the reference's dim_sp loop takes
    assert d["iterations"] == 939
    from diploma_research_gb300.generators import WORKLOADS

    assert d["config"] == bench._config(WORKLOADS["lap2d_512"]["build"]())
