"""The reference's own GA known answers (tests/test_gaboom.cpp) re-expressed against the host
decoder (flexaidds_gb300/system.py) and the GA restatement the device engine is checked against
(oracle/ga.py). The same answers are checked on the device in tests/test_gpu_ga_known_answers.py.

Each test names the reference test it re-expresses. The reference seeds its draws with srand or
random_device; here the draws are explicit sequences, chosen to cover what the reference's
assertions cover (e.g. "over 100 draws the dominant parent is chosen more than 90 times").
"""
import math

import numpy as np
import pytest

from flexaidds_gb300 import system
from oracle import ga

EPS = 1e-6


def seq(values):
    """A draw source that hands out the given uniforms in order."""
    it = iter(values)
    return lambda: next(it)


# --- RandomDouble / RandomInt (tests/test_gaboom.cpp:48-74) --------------------------------------

def test_random_double_mapping():
    assert system.random_double(0) == 0.0
    v = system.random_double(system.MAX_RANDOM_VALUE)
    assert 0.99 < v < 1.0
    assert abs(system.random_double(system.MAX_RANDOM_VALUE // 2) - 0.5) <= 0.01


def test_random_int_mapping():
    assert system.random_int(0.0) == 0
    assert system.random_int(1.0) == system.RAND_MAX


# --- genetoic / ictogene (tests/test_gaboom.cpp:80-135) ------------------------------------------
# The reference's fixture sets nbin = 11, bin = 1/11 on [0, 10] with del 1 by hand; set_bins gives
# exactly that for a mapped gene on those limits.

GL = dict(gmin=0.0, gmax=10.0, gdel=1.0, gmap=1)


def test_fixture_bins_are_set_bins_of_a_mapped_gene():
    assert system.bin_count(**GL) == 11.0
    tab = system.gene_bins(**GL)
    np.testing.assert_array_equal(tab[:11], np.cumsum(np.full(11, 1.0 / 11.0)))


def test_genetoic_in_range():
    tab = system.gene_bins(**GL)
    step = system.MAX_RANDOM_VALUE // 100
    for g in range(0, system.MAX_RANDOM_VALUE, step):
        ic = system.genetoic(tab, GL["gmin"], GL["gdel"], g)
        assert GL["gmin"] - EPS <= ic <= GL["gmax"] + EPS


@pytest.mark.parametrize("ic", [5.0, 0.0, 10.0])
def test_ictogene_round_trip(ic):
    tab = system.gene_bins(**GL)
    g = system.ic_to_gene(ic=ic, **GL)
    ic2 = system.genetoic(tab, GL["gmin"], GL["gdel"], g)
    assert GL["gmin"] - EPS <= ic2 <= GL["gmax"] + EPS
    if ic == 5.0:   # ICToGeneRoundTripsApproximately: within one bin of the original
        assert abs(ic2 - ic) <= GL["gdel"] + EPS


def test_descriptor_decoder_matches_genetoic():
    """The vectorised decoder of the descriptor (genes_to_ic) is genetoic gene by gene."""
    tab = system.gene_bins(**GL)
    genes = np.array([0, 1, 195225786, 195225787, 1 << 30, system.MAX_RANDOM_VALUE], np.int64)
    want = [system.genetoic(tab, 0.0, 1.0, int(g)) for g in genes]
    u = genes.astype(np.float64) / (2147483647.0 + 1.0)
    got = 0.0 + 1.0 * np.searchsorted(tab, u, side="left")
    np.testing.assert_array_equal(got, want)


# --- hash_genes (tests/test_gaboom.cpp:184-207) --------------------------------------------------

def test_hash_genes():
    assert ga.signature([1.0, 2.0, 3.0]) != ga.signature([1.0, 2.0, 4.0])
    assert ga.signature([5.0, 10.0]) == ga.signature([5.0, 10.0])
    assert ga.signature([7.3]) == ga.signature([7.3])


# --- remove_dups (tests/test_gaboom.cpp:309-372) --------------------------------------------------

@pytest.mark.parametrize("rows,kept", [
    ([[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]], 3),          # AllUnique
    ([[1.0, 2.0]] * 4, 1),                              # AllIdentical
    ([[1.0], [1.0], [5.0], [5.0]], 2),                  # SomeDuplicates
    ([[1.0, 2.0]], 1),                                  # SingleChromosome
    ([[1.0], [1.1]], 2),                                # ToleranceBoundary: 0.1 apart is not a duplicate
    ([[1.0], [1.05]], 1),                               # WithinTolerance
])
def test_remove_dups(rows, kept):
    assert len(ga.remove_dups(rows)) == kept


# --- fitness_stats (tests/test_gaboom.cpp:378-402) ------------------------------------------------

def test_fitness_stats():
    _, tot, mx, avg = ga.fitness_stats([10.0, 20.0, 30.0, 40.0])
    assert avg == 25.0 and mx == 40.0 and tot == 100.0
    _, _, _, avg1 = ga.fitness_stats([42.0])
    assert avg1 == 42.0


# --- adapt_prob (tests/test_gaboom.cpp:404-459) ---------------------------------------------------

def test_adapt_prob_high_fitness():
    crossp, mutp = ga.adapt_prob(100.0, 50.0, 80.0, 90.0, (1.0, 1.0, 0.5, 0.5))
    assert abs(crossp - 0.2) <= EPS and abs(mutp - 0.4) <= EPS


def test_adapt_prob_below_average():
    crossp, mutp = ga.adapt_prob(100.0, 50.0, 20.0, 30.0, (1.0, 1.0, 0.5, 0.3))
    assert crossp == 0.5 and mutp == 0.3


def test_adapt_prob_at_max():
    crossp, _ = ga.adapt_prob(100.0, 50.0, 100.0, 60.0, (1.0, 1.0, 0.5, 0.5))
    assert abs(crossp) <= EPS


# --- crossover (tests/test_gaboom.cpp:461-497) ----------------------------------------------------

def crossover_draws(rng, n):
    return [list(rng.random(8)) for _ in range(n)]


@pytest.mark.parametrize("intragenes", [False, True])
def test_crossover_conserves_material(intragenes):
    """MaterialIsConserved: every bit of both parents survives in one child or the other, for
    many draws (the reference checks one srand seed)."""
    rng = np.random.default_rng(42)
    for draws in crossover_draws(rng, 500):
        john = [0x0F0F0F0F, 0x00FF00FF]
        mary = [0xF0F0F0F0, 0xFF00FF00]
        before = [(j, m) for j, m in zip(john, mary)]
        ga.crossover(john, mary, intragenes, seq(draws))
        for (j0, m0), j, m in zip(before, john, mary):
            assert j | m == j0 | m0
            assert j & m == j0 & m0          # each bit position keeps its pair of values
            assert 0 <= j <= 0xFFFFFFFF and 0 <= m <= 0xFFFFFFFF


def test_crossover_single_gene_swaps_symmetrically():
    """SingleGeneSwapsBits: with one gene and crossover inside genes, both children change or
    neither does."""
    rng = np.random.default_rng(123)
    changed = 0
    for draws in crossover_draws(rng, 500):
        john, mary = [0xAAAAAAAA], [0x55555555]
        ga.crossover(john, mary, True, seq(draws))
        jc, mc = john[0] != 0xAAAAAAAA, mary[0] != 0x55555555
        assert jc == mc
        changed += jc
    assert changed > 400


# --- mutate (tests/test_gaboom.cpp:499-523) -------------------------------------------------------

def test_mutate_zero_rate():
    john = [0x12345678, 0xABCDEF01, 0x0]
    ga.mutate(john, 0.0, seq(np.random.default_rng(1).random(96)))
    assert john == [0x12345678, 0xABCDEF01, 0x0]


def test_mutate_full_rate():
    john = [0x00000000]
    ga.mutate(john, 1.0, seq(np.random.default_rng(2).random(32)))
    assert john == [0xFFFFFFFF]


# --- roulette_wheel (tests/test_gaboom.cpp:525-564) ----------------------------------------------

def test_roulette_uniform_fitness():
    f = ga.Fitness.given([1.0] * 5)
    for u in np.random.default_rng(42).random(50):
        assert 0 <= f.roulette(u) < 5


def test_roulette_dominant_fitness():
    f = ga.Fitness.given([0.001, 0.001, 1000.0])
    hits = sum(f.roulette(u) == 2 for u in np.random.default_rng(42).random(100))
    assert hits > 90


def test_roulette_single():
    assert ga.Fitness.given([5.0]).roulette(0.7) == 0


def test_roulette_first_running_sum_above():
    """roullete_wheel walks tot <= r: the index returned is the first whose running sum exceeds r."""
    f = ga.Fitness.given([1.0, 2.0, 3.0])
    assert f.roulette(0.0) == 0
    assert f.roulette(1.0 / 6.0) == 1            # r = 1.0 equals the first running sum
    assert f.roulette(0.5) == 2                  # r = 3.0 equals the second
    assert f.roulette(0.999) == 2


# --- calc_rmsp (tests/test_gaboom.cpp:566-590) ----------------------------------------------------

def test_calc_rmsp():
    assert abs(ga.calc_rmsp([1.0, 2.0, 3.0], [1.0, 2.0, 3.0])) <= EPS
    assert abs(ga.calc_rmsp([0.0, 0.0, 0.0], [1.0, 1.0, 1.0]) - 1.0) <= EPS
    assert abs(ga.calc_rmsp([3.0, 4.0], [0.0, 0.0]) - ga.calc_rmsp([0.0, 0.0], [3.0, 4.0])) <= EPS


def test_niche_counts_known_distance():
    """The niche count over (0,0,0) and (1,1,1) with sig_share 2: 1 + (1 - 1/2) each."""
    share = ga.niche_counts(np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]]), 2.0, 1.0)
    assert share == [1.5, 1.5]
    assert math.isclose(ga.niche_counts(np.array([[0.0], [3.0]]), 2.0, 1.0)[0], 1.0)
