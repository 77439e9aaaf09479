"""The multi-GPU form of the benchmark is N independent replicas: each rank
projects its own seeded scene, and the job's time is the slowest rank's.
This checks that host logic with two gloo ranks on the CPU (no GPU), and runs
each replica's data path there with the oracle: a rank projects the scene of
its own seed, with no collective on the data."""
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


def _replica_project(rank, world, port, out):
    import numpy as np

    import bench
    import oracle as O
    from flub_gb300 import scenes
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, _, w = bench.dist_env()
        seed = bench.replica_seed("dam256", r)
        ref = O.project(scenes.dam(16, seed, levels=3), dtype=np.float32)
        mine = (seed, int(ref["iters"]), bool(ref["converged"]), float(np.abs(ref["p"]).sum()))
        res = [None] * w
        dist.all_gather_object(res, mine)
        out[rank] = res
    finally:
        dist.destroy_process_group()


def test_two_replicas_project_their_own_scenes():
    """Each of two gloo ranks projects the 16^3 dam break of its replica seed
    with the FP32 oracle; the gathered results match single-process
    projections of the same seeds, and the two replicas differ."""
    import numpy as np

    import bench
    import oracle as O
    from flub_gb300 import scenes
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_replica_project, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
        res = dict(out)
    assert res[0] == res[1]  # every rank saw the same gathered list
    for rank, (seed, iters, conv, psum) in enumerate(res[0]):
        assert seed == bench.replica_seed("dam256", rank)
        ref = O.project(scenes.dam(16, seed, levels=3), dtype=np.float32)
        assert conv and iters == int(ref["iters"])
        assert psum == float(np.abs(ref["p"]).sum())
    assert res[0][0][3] != res[0][1][3]
