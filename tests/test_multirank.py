"""The N>1 bench path on CPU: two gloo ranks, each a replica of the workload
(no data-path collective); the timing reduction is the max over ranks and
the value counts every rank's bases."""
import os
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world)
    out[rank] = (ms, bench.aggregate_value(1_000_000, world, ms))
    dist.destroy_process_group()


def test_two_rank_reduction():
    world, port = 2, 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        ms, value = res[r]
        assert ms == pytest.approx(15.0)  # the slowest rank's time on every rank
        assert value == pytest.approx(2 * 1_000_000 / 15e-3)
