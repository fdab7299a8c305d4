"""The multi-GPU path of bench.py is replicas only (groups never exchange
data): every rank integrates its own copy of the workload, the job's time is
the slowest rank's, and the whole-job value counts every rank's cells. Its
host logic runs here as two gloo processes on the CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    seconds = bench.max_over_ranks(2.0 + rank, world)       # rank 1 is the slow one
    out.put((rank, seconds, bench.job_value(65536 * 120, world, seconds)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_whole_job():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in results] == [3.0, 3.0]
    assert all(r[2] == 65536 * 120 * 2 / 3.0 for r in results)


def test_single_process_time_is_its_own():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(1.5, 1) == 1.5
    assert bench.job_value(100, 1, 2.0) == 50.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Under torchrun only rank 0 times the reference's CPU path; the other
    ranks exit without work or output."""
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    monkeypatch.setattr(bench, "run_reference", lambda *a: pytest.fail("rank 1 ran the reference"))
    bench.main()
    assert capsys.readouterr().out == ""
