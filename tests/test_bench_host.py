"""The multi-rank host logic of bench.py on two gloo ranks (CPU).

Under torchrun every rank dedisperses its own beam and the job's time is the
slowest rank's; this checks the beam assignment, the MAX reduction and the
whole-job value without a GPU.
"""
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


def _rank(rank, world, port, result):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as tdist
    import bench
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        # rank r "took" 1.0 + r seconds
        t = bench.max_over_ranks(1.0 + r, tdist, "cpu")
        result[r] = (w, local, bench.beam_seed(r), t,
                     bench.job_value(w, 10, 2048, 24576, t))
    finally:
        tdist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_weak_value():
    world = 2
    with mp.Manager() as m:
        result = m.dict()
        mp.start_processes(_rank, args=(world, _free_port(), result), nprocs=world,
                           start_method="spawn", join=True)
        res = dict(result)
    assert sorted(res) == [0, 1]
    seeds = {res[r][2] for r in res}
    assert len(seeds) == world  # one distinct beam per rank
    for r in res:
        w, local, _, t, value = res[r]
        assert w == world and local == r
        assert t == pytest.approx(2.0)  # the slowest rank's time on every rank
        assert value == pytest.approx(world * 10 * 2048 * 24576 / 2.0)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.job_value(1, 4, 2, 3, 2.0) == 12.0
