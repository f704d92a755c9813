"""Replicas on several GPUs (bench.py under torchrun): the host side of the
N > 1 path on CPU with the gloo backend, world size 2.  Each replica times
its own run; the whole-job rate uses the slowest replica's time; the
reference arm runs on rank 0 only."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, world, port, times, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    ms = bench.max_over_ranks(times[rank], dist, "cpu")
    dist.barrier()
    out.put((rank, ms, bench.whole_job_rate(1000, world, ms)))
    dist.destroy_process_group()


def test_slowest_replica_sets_the_rate():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    times = [2.0, 5.0]  # ms per replica
    port = _free_port()
    procs = [ctx.Process(target=_replica, args=(r, 2, port, times, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [5.0, 5.0]
    assert all(r[2] == pytest.approx(2 * 1000 / 5e-3) for r in res)


def test_whole_job_rate():
    assert bench.whole_job_rate(500, 1, 250.0) == pytest.approx(2000.0)
    assert bench.whole_job_rate(500, 4, 250.0) == pytest.approx(8000.0)


def test_reference_arm_runs_on_rank0_only(monkeypatch):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.run_reference(None) is None  # returns before any work
