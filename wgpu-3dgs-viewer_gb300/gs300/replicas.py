"""Independent render replicas, one process per GPU.

Views of a scene are independent (each frame reads the resident records and writes its own
target), so N GPUs run N replicas with no data-path collective.  The process group is used
only around a timed region: a barrier before it, and a MAX over ranks of the elapsed time
after it, so that whole-job throughput = all units of all ranks / the slowest rank's time.

The group is NCCL on GPUs and gloo on CPU (the host-side logic is exercised with gloo).
"""
import os


class Replicas:
    """Rank, world size and local device of this process, read from the launcher's env."""

    def __init__(self, backend=None, env=None):
        env = os.environ if env is None else env
        self.rank = int(env.get("RANK", "0"))
        self.world = int(env.get("WORLD_SIZE", "1"))
        self.local = int(env.get("LOCAL_RANK", "0"))
        if not (0 <= self.rank < self.world):
            raise ValueError(f"RANK {self.rank} outside WORLD_SIZE {self.world}")
        self.backend = backend
        self._dist = None

    @property
    def leader(self):
        return self.rank == 0

    def scene_seed(self, base):
        """Each replica renders its own seeded scene (same sizes, independent content)."""
        return int(base) + self.rank

    def init(self):
        """Join the process group when world > 1; returns self."""
        if self.world > 1 and self._dist is None:
            import torch
            import torch.distributed as dist

            if self.backend == "nccl":
                dist.init_process_group("nccl", device_id=torch.device("cuda", self.local))
            else:
                dist.init_process_group(self.backend or "gloo")
            self._dist = dist
        return self

    def barrier(self):
        if self._dist is not None:
            self._dist.barrier()

    def max_over_ranks(self, x):
        """The largest value of x over all ranks (x a float)."""
        if self._dist is None:
            return float(x)
        import torch

        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def job_rate(self, units_per_rank, seconds_this_rank):
        """(whole-job units/s, slowest rank's seconds): every rank did units_per_rank."""
        slowest = self.max_over_ranks(seconds_this_rank)
        if slowest <= 0.0:
            raise ValueError("timed region took no time")
        return self.world * units_per_rank / slowest, slowest

    def close(self):
        if self._dist is not None:
            self._dist.destroy_process_group()
            self._dist = None
