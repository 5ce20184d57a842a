"""CPU checks of the DE restatement (the oracle of the device generation)."""
import numpy as np

from oracle import de


def test_permutations_are_rotations_of_one_shuffle():
    for gen in range(5):
        perm, coin = de.permutations(16, 3, seed=7, gen=gen)
        assert sorted(perm[0]) == list(range(16))
        for s in (1, 2):
            # each slice is the shuffled order rotated by a shift in 1..5
            shifts = [k for k in range(1, 16) if all(perm[s][j] == perm[0][(j - k) % 16]
                                                   for j in range(16))]
            assert len(shifts) == 1 and 1 <= shifts[0] <= 6


def test_trial_respects_bounds_and_formulas():
    rng = np.random.default_rng(0)
    P, nv = 12, 7
    pop = rng.uniform(-1e-7, 1e-7, (P, nv))
    mean = pop.mean(0)
    glo, ghi = np.full(nv, -5e-7), np.full(nv, 5e-7)
    ilo, ihi = np.full(nv, -1e-7), np.full(nv, 1e-7)
    for strategy in (0, 1, 2):
        t, org = de.trial(pop, pop[0], mean, glo, ghi, ilo, ihi, strategy, 0.7, 0.9, 3, 1)
        lo = np.maximum(mean + ilo, glo)
        hi = np.minimum(mean + ihi, ghi)
        assert np.all(t >= np.minimum(lo, org) - 1e-22) and np.all(t <= np.maximum(hi, org) + 1e-22)
    # rand/1 without crossover and wide bounds: x_r3 + F (x_r1 - x_r2)
    wide = np.full(nv, 1.0)
    t, _ = de.trial(pop, pop[0], mean, -wide, wide, -wide, wide, 0, 0.5, 1.0, 3, 2)
    perm, _ = de.permutations(P, 3, 3, 2)
    np.testing.assert_array_equal(t, pop[perm[2]] + 0.5 * (pop[perm[0]] - pop[perm[1]]))


def test_selection_is_greedy():
    rng = np.random.default_rng(1)
    pop, tri = rng.normal(size=(6, 3)), rng.normal(size=(6, 3))
    f, ft = rng.uniform(size=6), rng.uniform(size=6)
    p2, f2, bv, best, mean, _ = de.select(pop, f, tri, ft, 1e300, np.zeros(3))
    assert np.all(f2 == np.minimum(f, ft))
    assert bv == f2.min() and np.array_equal(best, p2[np.argmin(f2)])
