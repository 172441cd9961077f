"""Host logic of the multi-GPU path: independent run shards, one process per
GPU, no data-path collective.

A VlaPy run never exchanges data with another run, so N GPUs take N disjoint
shards of a sweep (weak scaling: each rank keeps its own 4096-run workload,
drawn with its own seed).  A single run is not split across GPUs: its
x-FFTs need every x and its v-FFTs every v, so a split would cost an
all-to-all transpose per step, and every workload here fits on one GPU.

The only collectives are for measurement: a barrier around the timed region,
the maximum of the ranks' times and the sum of the units they processed.
They run on NCCL on GPUs and on gloo in the CPU tests.
"""

from __future__ import annotations

import os

import torch
import torch.distributed as dist


def env():
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(world, backend=None):
    """Join the process group when there is more than one rank."""
    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))


def shard_seed(base_seed, rank):
    """Seed of a rank's own shard of the sweep (rank 0 keeps the base seed)."""
    return int(base_seed) + 7919 * int(rank)


def shard_runs(runs, rank, world):
    """Contiguous, disjoint shards covering every run (for a fixed global list)."""
    n = len(runs)
    lo = (n * rank) // world
    hi = (n * (rank + 1)) // world
    return runs[lo:hi]


def _device():
    if dist.is_initialized() and dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def barrier(world):
    if world > 1:
        dist.barrier()


def aggregate(ms, units, world):
    """(max time over ranks in ms, total units over ranks, units per second)."""
    if world == 1:
        return ms, units, units / (ms / 1e3)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=_device())
    u = torch.tensor([float(units)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    t_max, total = float(t.item()), float(u.item())
    return t_max, total, total / (t_max / 1e3)
