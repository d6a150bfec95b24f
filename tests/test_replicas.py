"""Multi-GPU form of the bench: replicas, one process per GPU, no collective on the data path; the job's time is
the slowest rank's and its work the sum over ranks (bench.reduce_replicas). Run here as two gloo ranks on CPU."""
import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, units = bench.reduce_replicas(dist, 10.0 + 5.0 * rank, 1000 * (rank + 1), "cpu")
    out[rank] = (ms, units)
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replicas_take_the_slowest_rank_and_sum_the_work():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert res == {0: (15.0, 3000), 1: (15.0, 3000)}
