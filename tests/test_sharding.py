"""The multi-rank path on the CPU (gloo, world size 2): slices partition the
batch, and differential evolution with replicated state and sharded
evaluation (costs all-gathered) follows the single-process run bit for bit
(the oracle's generation, the same counter-based draws on every rank)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from csim_gb300.sharding import ShardedObjective, max_over_ranks, shard_range
from oracle import de as ode


def test_max_over_ranks_without_group():
    assert max_over_ranks(3.25) == 3.25


def test_shard_range_partitions():
    for n in (0, 1, 5, 64, 65, 320):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = shard_range(n, r, world)
                assert 0 <= lo <= hi <= n
                seen += list(range(lo, hi))
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def _objective(x: torch.Tensor, out: torch.Tensor):
    # a deterministic per-candidate cost (a shifted sphere)
    out.copy_(((x - 0.1) ** 2).sum(1))


def _run_de(objective, P=10, nv=6, gens=6, seed=11):
    glo, ghi = -np.ones(nv), np.ones(nv)
    ilo, ihi = -np.ones(nv), np.ones(nv)
    pop = ode.init_uniform(P, np.zeros(nv), ilo, ihi, 1.0, seed)
    f = torch.empty(P, dtype=torch.float64)
    objective(torch.as_tensor(pop), f)
    f = f.numpy().copy()
    bi = int(np.argmin(f))
    best_val, best = float(f[bi]), pop[bi].copy()
    mean = pop.mean(0)
    for g in range(1, gens + 1):
        tri, _ = ode.trial(pop, best, mean, glo, ghi, ilo, ihi, 0, 0.7, 0.9, seed, g)
        ft = torch.empty(P, dtype=torch.float64)
        objective(torch.as_tensor(tri), ft)
        pop, f, best_val, best, mean, _ = ode.select(pop, f, tri, ft.numpy(), best_val, best)
    return pop, f, best_val


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pop, f, best = _run_de(ShardedObjective(_objective))
        slowest = max_over_ranks(10.0 + rank)  # a step timed per rank
        q.put((rank, pop, f, best, slowest))
    finally:
        dist.destroy_process_group()


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_de_matches_single_process():
    ref_pop, ref_f, ref_best = _run_de(_objective)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, pop, f, best, slowest in got:
        assert slowest == 10.0 + world - 1
        assert np.array_equal(pop, ref_pop), rank
        assert np.array_equal(f, ref_f), rank
        assert best == ref_best


class _ChainLikeObjective:
    """A CPU stand-in for optimize.PropagatedObjective with its call shape:
    a fixed batch of `pop` candidates whose sags are copied into the
    objective's own buffer (the chain's sag buffer) before evaluating, and
    a cost per candidate: here the response-matrix contrast of the oracle
    (optObjective.cpp:24-69) on a seeded matrix."""

    def __init__(self, pop, nvar, seed=3):
        rng = np.random.default_rng(seed)
        self.m = (rng.standard_normal((2, 40, nvar + 1))
                  + 1j * rng.standard_normal((2, 40, nvar + 1)))
        self.lam = np.array([6.3e-7, 6.7e-7])
        self.sags = torch.zeros((pop, nvar), dtype=torch.float64)
        self.pop = pop

    def __call__(self, x, out):
        if x.shape[0] != self.pop:
            raise ValueError("batch size differs from the chain's")
        self.sags.copy_(x)
        from oracle.elements import opt_hex_resp_objective
        v = opt_hex_resp_objective(self.m, self.lam, 1.0, self.sags.numpy().T * 1e-7)
        out.copy_(torch.as_tensor(np.asarray(v, np.float64).ravel()))
        return out


def _worker_chain(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = shard_range(10, rank, world)  # each rank's chain holds its slice
        pop, f, best = _run_de(ShardedObjective(_ChainLikeObjective(hi - lo, 6)))
        q.put((rank, pop, f, best))
    finally:
        dist.destroy_process_group()


def test_sharded_propagated_objective_matches_single_process():
    """ShardedObjective around an objective with PropagatedObjective's call
    shape: every rank builds its chain for its own slice of the population
    (shard_range), and the sharded DE equals one process evaluating the whole
    population with one chain."""
    ref_pop, ref_f, ref_best = _run_de(_ChainLikeObjective(10, 6))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_worker_chain, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, pop, f, best in got:
        assert np.array_equal(pop, ref_pop), rank
        assert np.array_equal(f, ref_f), rank
        assert best == ref_best


def test_sharded_objective_not_captured_in_generation_graph():
    """The all-gather stays outside captured graphs: GraphedGeneration
    refuses a ShardedObjective before touching the device."""
    from csim_gb300.optimize import GraphedGeneration
    sharded = object.__new__(ShardedObjective)
    with pytest.raises(ValueError, match="eager"):
        GraphedGeneration(None, "deRand1", sharded, None)
