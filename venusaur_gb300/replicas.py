"""Multi-process (one GPU per rank) helpers.

The path tracer shards without any data-path collective: pixels, samples and
whole jobs are independent.  On N GPUs each rank renders its own replica (or
its own share of a job list); the only communication is a barrier around the
timed region and a max-reduction of the elapsed time, so that the reported
throughput is (units of all ranks) / (slowest rank's time).

Ranks read RANK / WORLD_SIZE / LOCAL_RANK / MASTER_* from the environment
(torchrun).  NCCL is used when CUDA is available, gloo otherwise.
"""
from __future__ import annotations

import os


class Replicas:
    def __init__(self, backend: str | None = None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch
            import torch.distributed as dist

            if not dist.is_initialized():
                if backend is None:
                    backend = "nccl" if torch.cuda.is_available() else "gloo"
                dist.init_process_group(backend)
            self.dist = dist
            self.backend = dist.get_backend()
        else:
            self.backend = None

    def _device(self):
        import torch

        return torch.device("cuda", self.local) if self.backend == "nccl" else torch.device("cpu")

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def max(self, value: float) -> float:
        if self.dist is None:
            return float(value)
        import torch

        t = torch.tensor([float(value)], dtype=torch.float64, device=self._device())
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, value: float) -> float:
        if self.dist is None:
            return float(value)
        import torch

        t = torch.tensor([float(value)], dtype=torch.float64, device=self._device())
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def throughput(self, local_units: float, local_seconds: float) -> tuple[float, float, float]:
        """(units of all ranks, slowest rank's seconds, aggregate units/s)."""
        units = self.sum(local_units)
        secs = self.max(local_seconds)
        return units, secs, units / secs if secs > 0 else 0.0

    def shard(self, items):
        """This rank's share of a list of independent jobs (round robin)."""
        return list(items)[self.rank::self.world]

    def close(self) -> None:
        if self.dist is not None and self.dist.is_initialized():
            self.dist.destroy_process_group()
