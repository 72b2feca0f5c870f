"""Replicas across GPUs: the host logic of running one independent box per
rank (the step has no data-parallel split: a box needs global transposes and
a global CFL maximum, so N GPUs run N boxes, weak scaling).

One process per GPU (torchrun sets RANK, LOCAL_RANK, WORLD_SIZE); the only
communication is a barrier around the timed region and the maximum of the
ranks' times, so the whole-job throughput is N x cells x steps / max time.
NCCL on GPUs; the same calls run on gloo for the CPU tests.
"""
from __future__ import annotations

import os


def env():
    """(world, rank, local_rank) from the launcher's environment (1, 0, 0 without one)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Replicas:
    def __init__(self, backend: str = "nccl"):
        self.world, self.rank, self.local = env()
        self.dist = None
        self.backend = backend
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group(backend)
            self.dist = dist

    def seed(self, base: int = 0) -> int:
        """Each replica steps its own box: a seed per rank."""
        return base + self.rank

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def max(self, values):
        """Element-wise maximum over the ranks of a list of floats."""
        if self.dist is None:
            return [float(v) for v in values]
        import torch
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return [float(x) for x in t.cpu()]

    def throughput(self, cells_per_rank: int, steps: int, ms_local: float):
        """(whole-job cell-updates/s, the slowest rank's ms) for weak scaling."""
        (ms,) = self.max([ms_local])
        return self.world * cells_per_rank * steps / (ms * 1e-3), ms

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None
