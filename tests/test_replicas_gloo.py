"""The multi-GPU form of the benchmark is N independent replicas: each rank
projects its own seeded scene, and the job's time is the slowest rank's.
This checks that host logic with two gloo ranks on the CPU (no GPU)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, lr, w = bench.dist_env()
        local_ms = 10.0 + 5.0 * rank  # the slower rank sets the job's time
        job = bench.max_over_ranks(local_ms, w, "cpu")
        seed = bench.replica_seed("dam256", r)
        seeds = [None] * w
        dist.all_gather_object(seeds, seed)
        out[rank] = (r, w, job, bench.job_ms_per_projection(job, 4, w), seeds)
    finally:
        dist.destroy_process_group()


def test_two_replicas_time_and_seeds():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
        res = dict(out)
    for rank in range(world):
        r, w, job, per, seeds = res[rank]
        assert (r, w) == (rank, world)
        assert job == pytest.approx(15.0)               # max over ranks
        assert per == pytest.approx(15.0 / (4 * 2))     # whole job: steps x world projections
        assert len(set(seeds)) == world                  # every replica has its own scene
