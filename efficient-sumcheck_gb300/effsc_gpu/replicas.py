"""Replicas across GPUs of one node: one process per GPU, each proving its own
instances (the crate's proofs do not shard; there is no data-path
collective).  Only the measurement harness synchronises: a barrier around the
timed region, the maximum of the per-rank times, and the whole-job rate from
the units every rank processed.  Launched by torchrun (RANK / LOCAL_RANK /
WORLD_SIZE / MASTER_ADDR / MASTER_PORT from the environment)."""
import os


class Replicas:
    def __init__(self, backend=None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        self.backend = backend
        if self.world > 1:
            import torch
            import torch.distributed as dist
            self.backend = backend or ("nccl" if torch.cuda.is_available() else "gloo")
            if self.backend == "nccl":
                dist.init_process_group("nccl", device_id=torch.device("cuda", self.local))
            else:
                dist.init_process_group(self.backend)
            self.dist = dist

    def _device(self):
        import torch
        return torch.device("cuda", self.local) if self.backend == "nccl" else torch.device("cpu")

    def barrier(self):
        """All ranks here, and this rank's GPU work finished."""
        import torch
        if self.dist is not None:
            self.dist.barrier()
        if torch.cuda.is_available():
            torch.cuda.synchronize()

    def max(self, value):
        """The maximum of `value` over ranks (every rank gets it)."""
        if self.dist is None:
            return float(value)
        import torch
        t = torch.tensor([float(value)], dtype=torch.float64, device=self._device())
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, value):
        if self.dist is None:
            return float(value)
        import torch
        t = torch.tensor([float(value)], dtype=torch.float64, device=self._device())
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def replica_seed(base, rank):
    """Each replica proves its own seeded inputs."""
    return base + 7919 * rank


def job_rate(units_per_step, steps, world, max_ms):
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time (weak scaling: every rank does the same work)."""
    return world * steps * units_per_step / (max_ms * 1e-3)
