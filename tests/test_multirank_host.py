"""Multi-rank host logic on CPU (gloo, world size 2): the served stream is
partitioned by request index with no exchange on the data path, and the
bench reduces only (busy time, wall time) by max and request counts by sum —
the whole-job figures equal what one process computes from all ranks' parts."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


class _Req:
    def __init__(self, idx):
        self.idx = idx


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    reqs = [_Req(i) for i in range(101)]
    mine = bench.shard(reqs, rank, world)
    busy = torch.tensor([1.0 + rank, 2.0 + 3 * rank], dtype=torch.float64)
    dist.all_reduce(busy, op=dist.ReduceOp.MAX)
    n = torch.tensor([len(mine)], dtype=torch.float64)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    out[rank] = ([r.idx for r in mine], busy.tolist(), int(n.item()))
    dist.barrier()
    dist.destroy_process_group()


def test_stream_shards_partition_and_reduce():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
    idx0, busy0, n0 = out[0]
    idx1, busy1, n1 = out[1]
    assert sorted(idx0 + idx1) == list(range(101))
    assert not set(idx0) & set(idx1)
    assert busy0 == busy1 == [2.0, 5.0]
    assert n0 == n1 == 101
