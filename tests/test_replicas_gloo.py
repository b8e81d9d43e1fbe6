"""The N > 1 path of bench.py on CPU: ranks are independent replicas (no data-path collective);
the job time is the slowest rank's and the rate counts every rank's units.  Two `gloo` ranks."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        assert (r, w, local) == (rank, world, rank)
        # rank k renders 1000 units per step for 10 steps in (k + 1) seconds
        max_s, rate = bench.replica_rate(1000.0, 10, float(rank + 1))
        out[rank] = (max_s, rate)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replica_rate_over_gloo_ranks(world):
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        max_s, rate = res[rank]
        assert max_s == float(world)                     # the slowest rank's time
        assert rate == 1000.0 * 10 * world / float(world)  # all ranks' units over that time


def test_single_process_rate():
    import bench

    assert bench.replica_rate(500.0, 4, 2.0) == (2.0, 1000.0)
