"""Independent replicas of the solve, one process per GPU (torchrun / torch.distributed.run).

The solve has no multi-GPU decomposition: every rank runs the whole workload on its own GPU
and the ranks only agree on timing (a barrier on both sides of the timed region and the
maximum time over ranks).  NCCL is used when CUDA is available, gloo otherwise (the CPU
tests).
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Optional


@dataclass
class Group:
    world: int
    rank: int
    local: int
    dist: Optional[object]  # torch.distributed when world > 1
    backend: Optional[str]

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x: float) -> float:
        """The maximum of x over the ranks."""
        if self.dist is None:
            return x
        import torch

        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()


def init(backend: Optional[str] = None) -> Group:
    """The process group of the replicas, from RANK / LOCAL_RANK / WORLD_SIZE / MASTER_*."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world <= 1:
        return Group(1, 0, local, None, None)
    import torch
    import torch.distributed as dist

    if backend is None:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return Group(world, rank, local, dist, backend)


def whole_job_rate(world: int, cells: int, iterations_per_rank: int, t_max: float) -> float:
    """Cell-iterations per second of all ranks together: every rank ran `iterations_per_rank`
    iterations over `cells` cells; the job took the slowest rank's time."""
    return world * cells * iterations_per_rank / t_max
