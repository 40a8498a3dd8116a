"""Replicas: N independent systems, one per GPU, one process per GPU.

The path does not shard here (one domain, no halo exchange), so several GPUs
run independent replicas; the only cross-rank operations are the barrier
around the timed region and the reductions of the result: the slowest
rank's time and the total work. No collective touches the data path.
"""
from __future__ import annotations


class Replicas:
    """Barrier and max/sum reductions over the ranks of one job (torchrun
    environment); a single process needs no process group. `backend` is
    "nccl" (one GPU per rank) or "gloo" (CPU, for tests)."""

    def __init__(self, world: int, local: int = 0, backend: str = "nccl"):
        self.world = world
        self.backend = backend
        if world > 1:
            import torch
            import torch.distributed as td
            if backend == "nccl":
                torch.cuda.set_device(local)
            td.init_process_group(backend)
            self.td, self.torch = td, torch

    def _tensor(self, x: float):
        dev = "cuda" if self.backend == "nccl" else "cpu"
        return self.torch.tensor([x], device=dev, dtype=self.torch.float64)

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        t = self._tensor(x)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.world == 1:
            return x
        t = self._tensor(x)
        self.td.all_reduce(t)
        return float(t.item())

    def throughput(self, local_units: float, local_seconds: float) -> float:
        """Whole-job rate: the units all ranks processed over the slowest
        rank's time (weak scaling: each rank its own replica)."""
        return self.sum(local_units) / self.max(local_seconds)

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()
