"""Replica runs over ranks: one process per GPU, each with its own independent context.

The time-step path does not shard (one lattice, one GPU), so N GPUs run N independent
replicas; the only cross-rank operations are a start barrier and the maximum over ranks
of the timed duration, on CPU tensors over gloo.  No data-path collective exists.
Ranks are read from the torchrun environment (RANK, WORLD_SIZE, LOCAL_RANK); the
rendezvous address comes from MASTER_ADDR / MASTER_PORT.
"""
import os


class Replicas:
    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, value):
        """Maximum of a float over all ranks (every rank receives it)."""
        if not self.dist:
            return float(value)
        import torch
        t = torch.tensor([float(value)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def aggregate_rate(self, units_per_rank, seconds_max):
        """Whole-job throughput: the units all replicas processed over the slowest rank's time."""
        return units_per_rank * self.world / seconds_max

    def close(self):
        if self.dist:
            self.dist.barrier()
            self.dist.destroy_process_group()
            self.dist = None
