"""Multi-GPU replicas: parameter points are independent, so N GPUs each
evaluate their own share of a batch with their own resident copy of the
analysis; the only exchange is the host-side gather of B float64 results (no
collective on the data path).  One process per GPU, launched by torchrun."""
from __future__ import annotations

import os

import numpy as np


def dist_info():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(n: int, rank: int, world: int) -> slice:
    """Contiguous share of ``n`` points for ``rank``; sizes differ by at most one."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return slice(lo, lo + base + (1 if rank < extra else 0))


class ReplicaGroup:
    """Barrier, max-reduction of timings and gather of results across ranks."""

    def __init__(self, world: int, backend: str = "nccl"):
        self.world = world
        self.backend = backend
        if world > 1:
            import torch.distributed as td
            if not td.is_initialized():
                td.init_process_group(backend)
            self.td = td

    def _device(self):
        import torch
        return torch.device("cuda") if self.backend == "nccl" else torch.device("cpu")

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self._device())
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def gather(self, local: np.ndarray, n_total: int) -> np.ndarray:
        """Concatenate every rank's shard (rank order) into the full result."""
        if self.world == 1:
            return np.asarray(local)
        import torch
        rank = self.td.get_rank()
        sizes = [shard(n_total, r, self.world).stop - shard(n_total, r, self.world).start for r in range(self.world)]
        mx = max(sizes)
        buf = torch.zeros(mx, dtype=torch.float64, device=self._device())
        buf[:sizes[rank]] = torch.as_tensor(np.asarray(local), dtype=torch.float64)
        outs = [torch.zeros(mx, dtype=torch.float64, device=self._device()) for _ in range(self.world)]
        self.td.all_gather(outs, buf)
        return np.concatenate([o[:s].cpu().numpy() for o, s in zip(outs, sizes)])

    def close(self):
        if self.world > 1 and self.td.is_initialized():
            self.td.destroy_process_group()
