"""The N>1 bench path on CPU: two gloo ranks aggregate their replica timings the way bench.py
does under torchrun (slowest rank's time, sum of units)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from florence_gb300.replicas import job_throughput
    units = 1000.0 * (rank + 1)        # rank 0: 1000 elements, rank 1: 2000
    ms = 10.0 if rank == 0 else 20.0   # rank 1 is the slowest
    v, ms_max, total = job_throughput(units, ms)
    out[rank] = (v, ms_max, total)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replica_throughput():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        v, ms_max, total = out[r]
        assert ms_max == 20.0 and total == 3000.0
        assert abs(v - 3000.0 / 0.020) < 1e-6


def test_single_process_passthrough():
    from florence_gb300.replicas import job_throughput
    v, ms, u = job_throughput(500.0, 5.0)
    assert abs(v - 1e5) < 1e-9 and ms == 5.0 and u == 500.0
