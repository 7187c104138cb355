"""The multi-rank (replica) timing path of bench.py on CPU: two gloo ranks,
each with its own queries (seed 3 + rank); the job's time is the slowest
rank's (all-reduce MAX), and value = ranks x queries x submaps / time."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 + 5.0 * rank)
        from cmm_gpu.meshgen import random_sphere_points
        q = torch.from_numpy(random_sphere_points(8, seed=3 + rank))
        gathered = [torch.empty_like(q) for _ in range(world)]
        dist.all_gather(gathered, q)
        out[rank] = (ms, all(not torch.equal(gathered[0], g) for g in gathered[1:]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "cmm-s2_gb300"))
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0        # the slower rank's time on every rank
    assert res[0][1] and res[1][1]               # ranks draw different queries


def test_single_process_time_is_unchanged():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5) == 12.5
