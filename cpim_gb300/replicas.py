"""Replica bookkeeping for runs on several GPUs of one node.

The propagation path has no data exchange between GPUs: its units (SAC
sweeps, network instances, requests) are independent, so a run on N GPUs is N
independent replicas, one process per GPU. Only the bookkeeping is shared:
which units a rank takes, and the whole-job rate from every rank's count and
time (the slowest rank's time bounds the job). The same code runs over NCCL
(CUDA tensors) or gloo (CPU tensors)."""
from __future__ import annotations

import torch
import torch.distributed as dist


def shard(n_items: int, rank: int, world: int) -> range:
    """Contiguous, balanced slice of item indices for one rank (the first
    n_items % world ranks take one more)."""
    if world < 1 or not 0 <= rank < world or n_items < 0:
        raise ValueError("bad shard arguments")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def job_rate(units: float, seconds: float, device: str = "cpu") -> tuple[float, float, float]:
    """(units of all ranks, slowest rank's seconds, whole-job units/s).
    Collective over the default process group when one is initialised."""
    if dist.is_available() and dist.is_initialized():
        u = torch.tensor([float(units)], dtype=torch.float64, device=device)
        t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        units, seconds = float(u.item()), float(t.item())
    return units, seconds, (units / seconds if seconds > 0 else 0.0)
