"""The multi-GPU path of bench.py is replicas over the survey's systems: no
collective on the data path, the job's time is the slowest rank's.  Tested
here with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        ms = 100.0 + 50.0 * rank            # rank 1 is the slower one
        slowest = bench.max_over_ranks(ms, "cpu")
        out[rank] = (slowest, bench.whole_job_seconds_per_solve(slowest, 2, 4, world))
    finally:
        dist.destroy_process_group()


def test_replica_timing_two_ranks():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    # every rank sees the slowest rank's time; 2 steps x 4 systems x 2 ranks solves
    assert res[0][0] == res[1][0] == 150.0
    assert res[0][1] == pytest.approx(0.150 / 16)


def test_single_process_needs_no_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, "cpu") == 12.5
