"""The multi-GPU path is replicas only (one independent lattice per rank, no
data exchange): bench.py's whole-job figures come from one all-reduce over
the ranks.  Run here as two gloo ranks on the CPU."""
import os
import socket
import sys

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port,
                            rank=rank, world_size=world)
    try:
        # rank r: 1 + r ms per iteration, 100 - 10 r MLUPS end to end
        ms, e2e = bench.replica_totals(1.0 + rank, 100.0 - 10.0 * rank, world, dist, "cpu")
        out[rank] = (ms, e2e)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_totals_two_gloo_ranks():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        ms, e2e = out[r]
        assert ms == 2.0            # the slowest rank's time per iteration
        assert e2e == 2 * 90.0      # world x the slowest rank's rate


def test_replica_totals_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_totals(1.5, 80.0, 1) == (1.5, 80.0)
