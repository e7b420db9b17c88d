"""Replicas on one node: each rank traces its own disjoint range of flights (weak
scaling) with no collective on the data path; the only exchanges are the timing
reductions of the benchmark (slowest rank, summed work).

Flights are independent and their seeds and jitters come from their global
index, so the records of rank r's range equal the same range of one large
batch.  `bench.py --gpus N` runs one replica per GPU over NCCL; the CPU tests run
the same helpers as gloo ranks.
"""


def flight_range(n_per_rank, rank):
    """Global index offset of rank `rank` when every rank traces n_per_rank flights."""
    return rank * n_per_rank


class Reducer:
    """Timing reductions over the ranks of a process group (identity without one)."""

    def __init__(self, dist=None, device="cpu"):
        self.dist = dist
        self.device = device

    def _reduce(self, x, op):
        if self.dist is None:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        return self._reduce(x, None if self.dist is None else self.dist.ReduceOp.MAX)

    def sum(self, x):
        return self._reduce(x, None if self.dist is None else self.dist.ReduceOp.SUM)

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def throughput(self, units, seconds):
        """Whole-job rate: the units of every rank over the slowest rank's time."""
        return self.sum(units) / self.max(seconds)
