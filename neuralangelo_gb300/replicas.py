"""Multi-GPU runs as independent replicas.

Rays are independent, so every rank trains on its own batch with its own copy of the
field; nothing crosses ranks on the data path.  What the ranks share is the timing:
a barrier on both sides of the timed region, the slowest rank's time, and the
whole-job throughput (units summed over ranks / that time).  The launch follows
torchrun's environment (RANK, LOCAL_RANK, WORLD_SIZE, MASTER_ADDR / MASTER_PORT):
NCCL on GPUs, gloo on CPU processes.
"""
import os

import torch
import torch.distributed as dist


class ReplicaGroup:
    def __init__(self, backend=None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.backend = None
        if self.world > 1:
            if not dist.is_initialized():
                dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))
            self.backend = dist.get_backend()

    def _device(self):
        return torch.device("cuda", torch.cuda.current_device()) if self.backend == "nccl" else torch.device("cpu")

    def barrier(self):
        if self.world > 1:
            dist.barrier()

    def _reduce(self, v, op):
        if self.world == 1:
            return float(v)
        t = torch.tensor([float(v)], dtype=torch.float64, device=self._device())
        dist.all_reduce(t, op=op)
        return float(t)

    def max(self, v):
        """The largest value over ranks (the slowest rank's time)."""
        return self._reduce(v, dist.ReduceOp.MAX if self.world > 1 else None)

    def sum(self, v):
        return self._reduce(v, dist.ReduceOp.SUM if self.world > 1 else None)

    def throughput(self, units, seconds):
        """Whole-job rate: the units of every rank over the slowest rank's seconds."""
        return self.sum(units) / self.max(seconds)

    def close(self):
        if self.world > 1 and dist.is_initialized():
            dist.destroy_process_group()
