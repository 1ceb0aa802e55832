"""Replica parallelism for steady solves: one process per GPU, each solving its
own flow conditions on its own copy of the mesh, no exchange on the data path.

The solve shards by condition (the reference's SteadyFlowCase solves one
condition per run; conditions are independent), so N ranks run N independent
solves.  The only collective operations are the barrier around the timed
region and the maximum of the per-rank times, from which the whole-job
throughput is formed (units processed by all ranks / slowest rank's time).
"""
import os


def rank_info():
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Replicas:
    """Process-group handling for N replica ranks (NCCL on GPUs, gloo on CPU)."""

    def __init__(self, backend="nccl", device=None):
        self.rank, self.world, self.local = rank_info()
        self.device = device
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            kw = {"device_id": device} if backend == "nccl" and device is not None else {}
            dist.init_process_group(backend, **kw)
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max_over_ranks(self, x):
        """Largest value of x over all ranks (x itself with one rank)."""
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64,
                         device=self.device if self.device is not None and self.device.type == "cuda" else "cpu")
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank, seconds):
        """Whole-job rate: units of all ranks over the slowest rank's time."""
        return self.world * units_per_rank / self.max_over_ranks(seconds)

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None
