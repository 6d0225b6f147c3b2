"""The multi-GPU path is independent replicas (no data-path collective).

bench.py combines the replicas with two reductions: the max of the
per-rank times and the sum of the per-rank work.  This runs that code with
world_size 2 on the gloo backend on the CPU.
"""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import bench
    value, ms = bench.replica_throughput(torch, world, units_local=60.0, ms_local=100.0 * (rank + 1), device='cpu')
    q.put((rank, value, ms))
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms in out:
        assert ms == pytest.approx(200.0)              # slowest rank
        assert value == pytest.approx(120.0 / 0.2)     # 2 x 60 layers in 0.2 s


def test_single_rank_is_identity():
    import bench
    value, ms = bench.replica_throughput(torch, 1, 60.0, 120.0, device='cpu')
    assert ms == 120.0 and value == pytest.approx(500.0)
