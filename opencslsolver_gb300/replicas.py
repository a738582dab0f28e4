"""Replica groups for multi-GPU runs.

The linear-solve path does not shard: the triangular sweeps of the ILU factor
are a single dependency chain, and splitting them (block Jacobi) would change
the factor the reference defines.  N GPUs therefore run N independent
replicas of the same solve; the only collective work is a barrier around the
timed region and a max over ranks of the elapsed time, so the whole-job rate
is N x (one replica's rate) measured against the slowest rank.

One process per GPU, launched by torchrun (RANK, LOCAL_RANK, WORLD_SIZE,
MASTER_ADDR / MASTER_PORT in the environment).  The backend is NCCL on GPUs;
the same code runs over gloo on CPU, which is how it is tested.
"""
from __future__ import annotations

import os


class ReplicaGroup:
    def __init__(self, backend: str = "nccl", device=None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.device = device
        self._dist = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group(backend)
            self._dist = dist

    @property
    def is_root(self) -> bool:
        return self.rank == 0

    def barrier(self) -> None:
        if self._dist is not None:
            self._dist.barrier()

    def max_over_ranks(self, value: float) -> float:
        """The largest value over all ranks (the slowest rank's time)."""
        if self._dist is None:
            return float(value)
        import torch

        t = torch.tensor([float(value)], dtype=torch.float64, device=self.device)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def job_rate(self, ms_per_step: float) -> float:
        """Whole-job rate (per second) of `world` replicas, each taking
        ms_per_step (already the max over ranks) per step."""
        return self.world * 1000.0 / ms_per_step

    def close(self) -> None:
        if self._dist is not None:
            self._dist.destroy_process_group()
            self._dist = None
