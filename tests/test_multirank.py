"""Multi-GPU is replicas only: each rank runs its own commutators on its own
operators, and the ranks share only a barrier and the max of their timings.
This runs that host logic with two gloo ranks on the CPU: distinct replica
inputs, independent results (checked with the C oracle), the max-over-ranks
timing and the whole-job rate bench.py reports."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist
    import bench
    from oracle import Oracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sx, sy = bench.replica_seeds(rank)
    o = Oracle(2)
    X = o.ms.random_operator(sx, True)
    Y = o.ms.random_operator(sy, False)
    Z = o.commutator(X, Y, 1, -1)
    elapsed = 10.0 * (rank + 1)              # a slower second rank
    mx = bench.max_over_ranks(elapsed)
    dist.barrier()
    out[rank] = (float(np.linalg.norm(Z)), mx, bench.whole_job_value(world, 4, mx))
    dist.destroy_process_group()


def test_two_replicas_gloo():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
    (n0, m0, v0), (n1, m1, v1) = out[0], out[1]
    assert n0 != n1                          # independent replica inputs
    assert m0 == m1 == 20.0                  # max over ranks
    assert v0 == v1 == pytest.approx(2 * 4 / 0.020)
