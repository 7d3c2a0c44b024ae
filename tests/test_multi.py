"""Replica (weak-scaling) path of bench.py on CPU with the gloo backend.

Pairs are independent, so N GPUs run N independent batches with no
collective on the data path; the only cross-rank traffic is the final
max-of-times / sum-of-work reduction. This checks, with 2 gloo ranks, that
each rank draws its own shard of the workload and that the reductions give
whole-job numbers.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    w = bench.make_workload("plain_pairs", 6, rank)
    cells = bench.cells_full(w)
    t = 1.5 + rank  # stand-in per-rank step time
    out[rank] = (w.pairs[0][0].tobytes(), cells, bench.reduce_max(t, world),
                 bench.reduce_sum(cells, world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    r0, r1 = out[0], out[1]
    assert r0[0] != r1[0]                       # each rank aligns its own pairs
    assert r0[2] == r1[2] == 2.5                # slowest rank sets the time
    assert r0[3] == r1[3] == r0[1] + r1[1]      # whole-job cells
