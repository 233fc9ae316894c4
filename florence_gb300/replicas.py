"""Replica bookkeeping for multi-GPU runs.

Assembly shards over independent meshes (or element ranges) with no exchange on the data path,
so N GPUs run N independent replicas. The only cross-rank step is the timing: the job's time is
the slowest rank's, and the throughput is the units all ranks processed over that time.
"""
import torch
import torch.distributed as dist


def job_throughput(units_local, ms_local, device=None):
    """Returns (total units / max time [per second], max time in ms, total units) over all ranks.
    Works with any initialised process group (nccl: pass the rank's CUDA device; gloo: CPU)."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return units_local / (ms_local * 1e-3), ms_local, units_local
    dev = device if device is not None else torch.device("cpu")
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(units_local)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    ms = float(t.item())
    units = float(u.item())
    return units / (ms * 1e-3), ms, units
