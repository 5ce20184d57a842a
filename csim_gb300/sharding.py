"""Several GPUs, one process each: the batched path shards without a
data-path collective.

Fields ((wavelength, source, candidate) triples) are independent until the
contrast reduction, so ranks propagate disjoint batches. The one exchange is
in differential evolution (differentialEvolutionOptimizer.cpp:216-468): the
population and its counter-based random draws are replicated on every rank
(every rank generates the same trial vectors), each rank propagates its
contiguous slice of the trials, and the per-candidate costs (P values per
generation) are all-gathered, after which every rank's greedy selection is
identical. torch.distributed carries the exchange (NCCL for device tensors,
gloo for host tensors).
"""
from __future__ import annotations

import torch


def shard_range(n: int, rank: int, world: int) -> tuple:
    """The contiguous slice [lo, hi) of n items owned by `rank` of `world`:
    the first n % world ranks take one item more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def max_over_ranks(x: float, device="cpu", group=None) -> float:
    """The largest of the ranks' values of x (a timed region's length: the
    job is as slow as its slowest rank); x itself without a process group."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


class ShardedObjective:
    """objective(x, out) evaluated on this rank's slice of the candidates x
    [n][nvar], the costs all-gathered into out [n] on every rank."""

    def __init__(self, objective, group=None):
        import torch.distributed as dist
        self.objective, self.group, self.dist = objective, group, dist
        self.world = dist.get_world_size(group)
        self.rank = dist.get_rank(group)

    def __call__(self, x: torch.Tensor, out: torch.Tensor) -> torch.Tensor:
        n = x.shape[0]
        per = -(-n // self.world)  # equal padded slices for all_gather
        lo, hi = shard_range(n, self.rank, self.world)
        local = torch.zeros(per, dtype=out.dtype, device=out.device)
        if hi > lo:
            self.objective(x[lo:hi], local[:hi - lo])
        gathered = torch.empty(per * self.world, dtype=out.dtype, device=out.device)
        self.dist.all_gather_into_tensor(gathered, local, group=self.group)
        for r in range(self.world):  # unpad: rank r's values sit at [r per, r per + count)
            rl, rh = shard_range(n, r, self.world)
            out[rl:rh] = gathered[r * per:r * per + (rh - rl)]
        return out
