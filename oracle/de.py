"""FP64 restatement of the reference's differential evolution generation
(differentialEvolutionOptimizer.cpp:216-468, deStrategy.cpp:23-158) with the
counter-based random generator the GPU kernels use, so a generation can be
compared bit for bit.

TEST INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import numpy as np

M64 = (1 << 64) - 1
RS_SHUF1, RS_SHUF2, RS_COIN, RS_CROSS, RS_BOUNCE, RS_INIT = 1, 2, 3, 4, 5, 6


def splitmix64(z: int) -> int:
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def uniform(seed: int, gen: int, stream: int, idx: int) -> float:
    k = splitmix64(seed & M64)
    k = splitmix64(k ^ (gen & M64))
    k = splitmix64(k ^ ((stream << 56) & M64) ^ (idx & M64))
    return (k >> 11) * (1.0 / 9007199254740992.0)


def permutations(P: int, n_slices: int, seed: int, gen: int):
    """makePopulationPermutations (deStrategy.cpp:23-65): slice 0 = a
    shuffle si1 of the candidates; slice s+1 = slice s rotated by
    si2(s) + 1, si2 a shuffle of 0..n_slices-1. Returns [n_slices][P] and the
    either-or coin (eitherOr's rand() < 0.5, deStrategy.cpp:125)."""
    si1 = list(range(P))
    for i in range(P - 1, 0, -1):
        j = int(uniform(seed, gen, RS_SHUF1, i) * (i + 1))
        si1[i], si1[j] = si1[j], si1[i]
    si2 = [0, 1, 2]
    for i in range(n_slices - 1, 0, -1):
        j = int(uniform(seed, gen, RS_SHUF2, i) * (i + 1))
        si2[i], si2[j] = si2[j], si2[i]
    perm = [si1]
    shift = 0
    for s in range(1, n_slices):
        shift += si2[s - 1] + 1
        perm.append([si1[(j - shift) % P] for j in range(P)])
    coin = uniform(seed, gen, RS_COIN, 0) < 0.5
    return np.array(perm), coin


def trial(pop, best, mean, glo, ghi, ilo, ihi, strategy, fw, cr, seed, gen):
    """Mutation, binomial crossover (:360-369) and bounce-back (:395-434).
    pop is [P][nvar]; strategy 0 rand/1, 1 local-to-best/1, 2 either-or."""
    P, nv = pop.shape
    perm, coin = permutations(P, 2 if strategy == 1 else 3, seed, gen)
    out = np.empty_like(pop)
    org = np.empty_like(pop)
    for c in range(P):
        for v in range(nv):
            i = c * nv + v
            x = pop[c, v]
            a = pop[perm[0][c], v]
            b = pop[perm[1][c], v]
            if strategy == 1:
                mut = (x + fw * (best[v] - x)) + fw * (a - b)
                orig = x
            else:
                base = pop[perm[2][c], v]
                if strategy == 0 or coin:
                    mut = base + fw * (a - b)
                else:
                    k = 0.5 * (fw + 1.0)
                    mut = base + k * ((a + b) - 2.0 * base)
                orig = base
            cand = mut
            if cr < 1.0 and not (uniform(seed, gen, RS_CROSS, i) < cr):
                cand = x
            up = min(mean[v] + ihi[v], ghi[v])
            lo = max(mean[v] + ilo[v], glo[v])
            if cand < lo:
                cand = lo + uniform(seed, gen, RS_BOUNCE, i) * (orig - lo)
            elif cand > up:
                cand = up + uniform(seed, gen, RS_BOUNCE, i) * (orig - up)
            out[c, v] = cand
            org[c, v] = orig
    return out, org


def select(pop, f, tri, f_tri, best_val, best):
    """Greedy selection (:436-453), best member (:371-393) and the population
    mean (sequential sum, compute_population_statistics)."""
    pop = pop.copy()
    f = f.copy()
    better = f_tri < f
    pop[better] = tri[better]
    f[better] = f_tri[better]
    bi = int(np.argmin(f))
    best = best.copy()
    if f[bi] < best_val:
        best_val = float(f[bi])
        best = pop[bi].copy()
    mean = np.zeros(pop.shape[1])
    for c in range(pop.shape[0]):
        mean = mean + pop[c]
    mean = mean / pop.shape[0]
    dist = np.sqrt(((pop - mean) ** 2).sum(1))
    return pop, f, best_val, best, mean, (dist.mean(), dist.max())


def init_uniform(P, origin, ilo, ihi, spread, seed, gen=0):
    """init_population (:336-358), uniform: origin + spread (u - 1/2) (UB - LB)."""
    nv = origin.size
    out = np.empty((P, nv))
    for c in range(P):
        for v in range(nv):
            i = c * nv + v
            r = uniform(seed, gen, RS_INIT, i) - 0.5
            out[c, v] = origin[v] + (spread * r) * (ihi[v] - ilo[v])
    return out
