"""Independent replicas of a workload on the GPUs of one node.

The unsplit step of one run has no exchange with another run, so N GPUs run
N replicas (the ensemble already batches independent runs on one GPU).  This
is the host side of that: process-group setup from the torchrun environment
(RANK, WORLD_SIZE, LOCAL_RANK, MASTER_ADDR/PORT), a barrier, the maximum of a
timing over ranks (the slowest replica times the job), and the whole-job
rate.  The only collectives are these scalars, on the gloo backend.
"""

from __future__ import annotations

import os


class Replicas:
    def __init__(self, backend: str = "gloo"):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x: float) -> float:
        """The largest value of x over the ranks (every rank gets it)."""
        if self.dist is None:
            return float(x)
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def total_rate(self, units_per_rank: float, ms: float) -> float:
        """Whole-job rate in units per second: every rank processed
        units_per_rank in its own ms; the job lasts the slowest rank's time."""
        return units_per_rank * self.world / (self.max(ms) / 1e3)

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None
