"""The multi-rank logic of bench.py on CPU: world_size 2 over gloo.

Each rank runs an independent replica; the job's time is the slowest rank's
(max over ranks) and the job's throughput counts every rank's cells.  The
reference arm runs on rank 0 alone and the other ranks exit without work.
"""
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


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = [12.5, 30.0][rank]
        t = bench.max_over_ranks(local_ms, world)
        q.put((rank, t, bench.job_mlups(1000, 10, world, t * 1e-3)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_value():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [30.0, 30.0]
    # 2 ranks x 1000 cells x 10 steps in 30 ms
    assert all(abs(g[2] - 2 * 1000 * 10 / 0.030 / 1e6) < 1e-9 for g in got)


def test_single_rank_time_is_local():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(7.0, 1) == 7.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    called = []
    monkeypatch.setattr(bench, "time_cpu_oracle", lambda *a, **k: called.append(1))
    assert bench.run_reference(bench.parse_args(["--impl", "reference", "--gpus", "2"])) == 0
    assert not called and capsys.readouterr().out == ""
