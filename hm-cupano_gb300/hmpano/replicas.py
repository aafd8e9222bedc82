"""Replicas across GPUs: one stitcher per rank, one GPU per rank, and no exchange of data (frames,
streams and requests are independent). A timed region is bracketed by barriers, the time per
step is the maximum over ranks (the slowest replica bounds the job), and the job's throughput is
the units every rank processed over that time.

The process group comes from the torchrun environment (RANK, WORLD_SIZE, LOCAL_RANK, MASTER_ADDR,
MASTER_PORT); with WORLD_SIZE 1 no group is made and every call is local.
"""
from __future__ import annotations

import os


class Replicas:
    def __init__(self, rank: int, world: int, local: int, dist=None, device=None):
        self.rank, self.world, self.local = rank, world, local
        self._dist, self._device = dist, device

    def barrier(self) -> None:
        if self._dist is not None:
            self._dist.barrier()

    def max_over_ranks(self, value: float) -> float:
        """The largest `value` of any rank (every rank gets it)."""
        if self._dist is None:
            return float(value)
        import torch

        t = torch.tensor([float(value)], dtype=torch.float64, device=self._device)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def job_rate(self, units_per_rank: float, seconds: float) -> float:
        """Units per second of the whole job: every rank processed `units_per_rank` in `seconds`."""
        return self.world * units_per_rank / seconds

    def close(self) -> None:
        if self._dist is not None:
            self._dist.destroy_process_group()
            self._dist = None


def init(backend: str = "nccl") -> Replicas:
    """Join the process group of a multi-rank launch ("nccl": one CUDA device per rank, bound to
    LOCAL_RANK; "gloo": CPU, for tests)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world <= 1:
        return Replicas(rank, 1, local)
    import torch
    import torch.distributed as dist

    if backend == "nccl":
        device = torch.device("cuda", local)
        dist.init_process_group("nccl", device_id=device)
    else:
        device = torch.device("cpu")
        dist.init_process_group(backend)
    return Replicas(rank, world, local, dist, device)
