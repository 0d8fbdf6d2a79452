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


def _responses(O, f, nrec):
    import numpy as np
    rng = np.random.default_rng(100 + f)
    rows = []
    for _ in range(nrec):
        e0, h0, e1, h1 = (rng.standard_normal(3) + 1j * rng.standard_normal(3) for _ in range(4))
        rows.append(O.mt_response(e0, h0, e1, h1, 2 * np.pi * (f + 1)))
    return np.stack(rows)


def _survey_rank(rank, world, port, out):
    """One rank of a survey split across GPUs (calc.run under
    torch.distributed): it takes its block of frequencies, computes their MT
    responses (the oracle's impedance solve on seeded fields stands in for
    the GPU solve here) and the responses are gathered on rank 0."""
    import sys
    import numpy as np
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from mtcalc_with_dfp_cocr_gb300 import calc
    from oracle import pyoracle as O
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        nf, nrec = 7, 3
        idx = calc.rank_frequencies(nf, rank, world)
        local = np.stack([_responses(O, f, nrec) for f in idx]) if idx else np.zeros((0, nrec, 34))
        full = calc.gather_responses(local, idx, nf)
        out[rank] = (idx, None if full is None else full.tolist())
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_survey_split_across_ranks_gathers_every_frequency(world):
    import sys
    import numpy as np
    sys.path.insert(0, ROOT)
    from oracle import pyoracle as O
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_survey_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    # the blocks cover the frequencies once, in order; rank 0 holds them all
    assert sum((res[r][0] for r in range(world)), []) == list(range(7))
    assert all(res[r][1] is None for r in range(1, world))
    single = np.stack([_responses(O, f, 3) for f in range(7)])
    np.testing.assert_array_equal(np.array(res[0][1]), single)
