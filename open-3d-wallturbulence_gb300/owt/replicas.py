"""Replica runs over several GPUs: one independent channel per rank.

The time step does not exchange data between ranks here (each GPU advances
its own channel), so the only cross-rank operations are a barrier around the
timed region and the reduction of the per-rank times: the slowest rank sets
the wall time, and the aggregate rate counts every rank's steps.
"""
import torch
import torch.distributed as dist


def aggregate(local_ms, steps_per_rank, device=None):
    """Max-over-ranks time (ms) and whole-job rate (steps/s)."""
    world = dist.get_world_size() if dist.is_initialized() else 1
    ms = float(local_ms)
    if world > 1:
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * steps_per_rank * 1e3 / ms


def barrier(device_sync=True):
    if dist.is_initialized():
        dist.barrier()
    if device_sync and torch.cuda.is_available():
        torch.cuda.synchronize()
