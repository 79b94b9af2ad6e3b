"""Multi-rank paths of bench.py on CPU: world_size 2 over gloo (127.0.0.1).

Every rank renders the whole frame (replicas, weak scaling; the path has no
exchange step), so the only cross-rank operation is the element-wise maximum
of the timings, and the job throughput is all ranks' paths over that maximum.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    times = [1.0 + rank, 10.0 - rank, 0.5 * (rank + 1)]
    got = bench.reduce_over_ranks(times, world, "cpu")
    out[rank] = got
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_over_ranks_takes_the_slowest_replica():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        assert out[r] == [2.0, 10.0, 1.0]


def test_job_throughput_counts_every_replica():
    import bench
    paths = 1920 * 1080 * 16
    one = bench.job_throughput(paths, 5, 1, 0.2)
    two = bench.job_throughput(paths, 5, 2, 0.2)
    assert two == pytest.approx(2 * one)
    assert one == pytest.approx(paths * 5 / 0.2 / 1e6)


def test_reference_arm_prints_only_on_rank_zero(capsys, monkeypatch):
    import bench

    class Args:
        steps, warmup, gpus = 1, 0, 2
    bench.run_reference(Args, 2, 1)
    assert capsys.readouterr().out == ""
