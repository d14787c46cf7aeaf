"""The multi-GPU form of the benchmark is replicas: every rank renders its
own poses on its own copy of the DAG and only the timings and ray counts are
reduced (max of times, sum of rays).  This runs that host logic with two
gloo ranks on CPU."""
import os
import socket

import torch.multiprocessing as mp
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), HD_BENCH_GLOO="1")
    import bench
    dist = bench.Dist()
    assert dist.world == world and dist.rank == rank
    ms = 10.0 + rank          # this rank's device time
    rays = 1000 * (rank + 1)  # rays it traced
    total_ms = dist.max(ms)
    rays_all = dist.sum(rays)
    poses = [bench.replica_poses(k, 4, rank, 64) for k in range(4)]
    dist.barrier()
    out[rank] = (total_ms, rays_all, poses)
    dist.pg.destroy_process_group()


def test_two_gloo_replicas_reduce_timings_and_rays():
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    (m0, s0, p0), (m1, s1, p1) = out[0], out[1]
    assert m0 == m1 == 11.0          # max over ranks
    assert s0 == s1 == 3000.0        # whole-job rays
    assert p0 != p1                  # each replica renders its own poses
    assert all(len(set(step)) == 4 for step in p0 + p1)
