"""Multi-rank host logic of bench.py on CPU: two gloo ranks (world size 2).

The path has no exchange step, so N GPUs run N independent replicas; the only
cross-rank work is the barrier and the max-over-ranks time.  These tests run
that logic with the gloo backend on CPU (the same functions bench.py calls
with NCCL on GPUs).
"""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = bench.dist_setup()
        assert (w, r, local) == (world, rank, rank)
        dist.barrier()
        t = bench.max_over_ranks(times[rank], dist, torch.device("cpu"))
        out[rank] = t
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("times", [[1.5, 2.5], [3.0, 0.25]])
def test_max_over_ranks_gloo(times):
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, times, out), nprocs=world, join=True)
        got = dict(out)
    assert got == {0: max(times), 1: max(times)}


def test_whole_job_aggregate():
    # two replicas of 200 MB each, slowest replica at 0.1 ms per step
    assert bench.whole_job_gbs(200_000_000, 2, 0.1) == pytest.approx(4000.0)
    assert bench.whole_job_gbs(200_000_000, 1, 0.1) == pytest.approx(2000.0)
    assert bench.max_over_ranks(1.25) == 1.25


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class Args:
        workload = "cfg1"

    assert bench.run_reference_arm(Args()) == 0
