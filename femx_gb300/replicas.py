"""Replica-only multi-GPU execution (one process per GPU).

The assembly path shards by elements, but every instance here runs whole on
one GPU: under torchrun each rank runs its own copy of the workload (weak
scaling) with no data-path collective. The only collectives are for
measurement: a barrier around timed regions and a MAX over ranks of the
elapsed time, so the whole-job rate is (units per rank x ranks) / slowest
rank. Works over NCCL (CUDA tensors) and gloo (CPU tensors).
"""
from __future__ import annotations

import os

__all__ = ["Replicas"]


class Replicas:
    def __init__(self, dist=None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.dist = dist if self.world > 1 else None

    @property
    def reporter(self) -> bool:
        """Rank 0 prints the result line."""
        return self.rank == 0

    def _tensor(self, x):
        import torch
        dev = "cuda" if self.dist.get_backend() == "nccl" else "cpu"
        return torch.tensor([float(x)], dtype=torch.float64, device=dev)

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max_time(self, seconds: float) -> float:
        """The slowest rank's time (every rank gets it)."""
        if self.dist is None:
            return float(seconds)
        t = self._tensor(seconds)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def job_rate(self, units_per_rank: float, seconds: float) -> float:
        """Whole-job throughput: all ranks' units over the slowest time."""
        return units_per_rank * self.world / self.max_time(seconds)
