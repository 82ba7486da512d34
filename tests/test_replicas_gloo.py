"""The multi-GPU form is replicas: one simulation per rank, no collective on
the data path; the job's figures are the slowest rank's time and the summed
cell-steps (bench.aggregate_over_ranks).  Exercised here with two gloo ranks
on CPU, as a torchrun launch would run them."""
import os
import sys
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t, c = bench.aggregate_over_ranks(1.5 + rank, 1000 * (rank + 1), "cpu")
        out[rank] = (t, c)
    finally:
        dist.destroy_process_group()


def test_two_replicas_aggregate_max_time_and_summed_cell_steps():
    mgr = mp.Manager()
    out = mgr.dict()
    port = 29400 + (os.getpid() % 500)
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1] == (2.5, 3000.0)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert not dist.is_initialized()
    assert bench.aggregate_over_ranks(0.25, 42, "cpu") == (0.25, 42.0)
