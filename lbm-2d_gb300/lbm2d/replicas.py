"""Independent replicas across GPUs (one process per GPU, launched by
torchrun).  The D2Q9 step has no data-path exchange between replicas: each
rank runs its own solve; the only collectives are the timing barrier and the
max-over-ranks of the measured time, carried on the CPU (gloo) so no GPU
collective is involved."""
from __future__ import annotations

import os


def world():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class Replicas:
    def __init__(self):
        self.rank, self.size, self.local = world()
        self.dist = None
        if self.size > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, value: float) -> float:
        """Largest value over all ranks (the slowest replica's time)."""
        if not self.dist:
            return float(value)
        import torch
        t = torch.tensor([float(value)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t[0])

    def sum(self, value: float) -> float:
        if not self.dist:
            return float(value)
        import torch
        t = torch.tensor([float(value)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t[0])

    def close(self):
        if self.dist and self.dist.is_initialized():
            self.dist.destroy_process_group()
