"""The reference's GA known answers (tests/test_gaboom.cpp) on the device: the GA engine's breeding
code driven by fixed draws (fxe_ga_breed_draws), its niche-count kernel (fxe_ga_niche_counts)
and the device gene decoder (fxe_decode_genes), through the C ABI. The same answers are checked
against the host decoder and oracle/ga.py in tests/test_ga_known_answers.py; here the device is
also compared with oracle/ga.py operator by operator on random draws, bit for bit."""
import numpy as np
import pytest

from flexaidds_gb300 import evaluator, system
from oracle import ga

pytestmark = pytest.mark.gpu

EPS = 1e-6
NO_MUT = 0.99     # a draw above every mutation probability used here


def rows(ng, n, fill=NO_MUT):
    return np.full((n, evaluator.ga_draws_per_pair(ng)), fill, np.float64)


def breed(pop, fitness, draws, **kw):
    return evaluator.ga_breed_draws(pop, fitness, draws, **kw)


# --- genetoic / ictogene on the device decoder (tests/test_gaboom.cpp:80-135) --------------------

@pytest.fixture(scope="module")
def decoder(tiny_system):
    """The tiny system with one dihedral gene on the reference fixture's limits: [0, 10], del 1,
    nbin 11 (a mapped gene, as set_bins counts it)."""
    _, d0 = tiny_system
    d = system.Descriptor.from_arrays(d0.to_arrays())
    q = int(np.nonzero(d.gene_typ == 2)[0][0])
    d.gene_min[q], d.gene_max[q], d.gene_del[q], d.gene_map[q] = 0.0, 10.0, 1.0, 1
    d.decode = None
    ev = evaluator.GPUEvaluator(d, max_poses=64)
    yield d, q, ev
    ev.close()


def test_device_genetoic_in_range_and_round_trip(decoder):
    d, q, ev = decoder
    step = system.MAX_RANDOM_VALUE // 100
    g = np.zeros((101, d.n_genes), np.int32)
    g[:, q] = np.arange(0, system.MAX_RANDOM_VALUE, step)[:101]
    ic = ev.decode_genes(g)[:, q]
    assert np.all(ic >= -EPS) and np.all(ic <= 10.0 + EPS)
    for x in (5.0, 0.0, 10.0):
        gg = np.zeros((1, d.n_genes), np.int32)
        gg[0, q] = system.ic_to_gene(0.0, 10.0, 1.0, 1, x)
        back = ev.decode_genes(gg)[0, q]
        assert -EPS <= back <= 10.0 + EPS
        if x == 5.0:
            assert abs(back - x) <= 1.0 + EPS


def test_device_decoder_equals_host(decoder):
    d, _, ev = decoder
    rng = np.random.default_rng(3)
    g = rng.integers(0, 2 ** 31, size=(4000, d.n_genes), dtype=np.int64).astype(np.int32)
    g[0, :] = 0
    g[1, :] = system.MAX_RANDOM_VALUE
    np.testing.assert_array_equal(ev.decode_genes(g), d.genes_to_ic(g))
    np.testing.assert_array_equal(ev.decode_genes(g, clamp=True),
                                  np.clip(d.genes_to_ic(g), d.gene_min, d.gene_max))


# --- fitness_stats (tests/test_gaboom.cpp:378-402) ------------------------------------------------

def test_device_fitness_stats():
    pop = np.arange(8, dtype=np.int64).reshape(4, 2)
    r = breed(pop, [10.0, 20.0, 30.0, 40.0], rows(2, 1), cross_rate=0.0, mut_rate=0.0)
    assert r["mean"] == 25.0 and r["max"] == 40.0 and r["total"] == 100.0
    r1 = breed(pop[:1], [42.0], rows(2, 1), cross_rate=0.0, mut_rate=0.0)
    assert r1["mean"] == 42.0


# --- adapt_prob (tests/test_gaboom.cpp:404-459): seen through what the children do ----------------

FIT = [90.0, 80.0, 100.0, 0.0, 0.0, 30.0]     # max 100, mean 50; positions 0 and 1 hold 90 and 80
POP = np.array([[0x0F0F0F0F, 0x00FF00FF], [0xF0F0F0F0, 0xFF00FF00], [1, 1], [2, 2], [3, 3], [4, 4]], np.int64)


def adaptive_pair(k, cross_draw, mut_draw, pos=(0.1, 0.4)):
    """Parents at roulette positions 0 and 1 (r = 30 and 120 of 300); crossover of genes 0..1 at
    the gene boundary if cross_draw is under the crossover probability; the first bit draw of
    each child's first gene is mut_draw."""
    ng = 2
    d = rows(ng, 1)
    d[0, 0], d[0, 1], d[0, 2] = pos[0], pos[1], cross_draw
    # genes 0 and 1, points 0 and 32; none of these draws mutates a bit if they are read as
    # mutation draws (no crossover)
    d[0, 3], d[0, 4], d[0, 5], d[0, 6] = 0.45, 0.9, 0.9, 0.45
    r = breed(POP, FIT, d, cross_rate=0.0, mut_rate=0.0, adaptive=True, k=k)
    crossed = not np.array_equal(r["children"][:2], POP[:2] & 0xFFFFFFFF)
    d2 = rows(ng, 1)
    d2[0, :3] = (pos[0], pos[1], 1.0)                          # no crossover
    d2[0, 3] = mut_draw
    r2 = breed(POP, FIT, d2, cross_rate=0.0, mut_rate=0.0, adaptive=True, k=k)
    mutated = int(r2["children"][0, 0]) != (int(POP[0, 0]) & 0xFFFFFFFF)
    return crossed, mutated


def test_device_adapt_prob_high_fitness():
    k = (1.0, 1.0, 0.5, 0.5)                     # crossp 0.2, mutp 0.4
    assert adaptive_pair(k, 0.19, 0.39) == (True, True)
    assert adaptive_pair(k, 0.21, 0.41) == (False, False)


def test_device_adapt_prob_below_average():
    k = (1.0, 1.0, 0.5, 0.3)                     # both parents below the mean: crossp k3, mutp k4
    fit = [20.0, 30.0, 100.0, 50.0, 50.0, 50.0]  # max 100, mean 50; positions 0, 1 hold 20, 30
    d = rows(2, 1)
    d[0, :3] = (0.01, 0.1, 0.49)                 # r = 3 -> 0, r = 30 -> 1; crossp k3 = 0.5
    d[0, 3:7] = (0.45, 0.9, 0.9, 0.45)           # above mutp 0.3 when read as mutation draws
    crossed = not np.array_equal(breed(POP, fit, d, cross_rate=0.0, mut_rate=0.0, adaptive=True, k=k)["children"][:2],
                                 POP[:2] & 0xFFFFFFFF)
    d[0, 2] = 0.51
    kept = np.array_equal(breed(POP, fit, d, cross_rate=0.0, mut_rate=0.0, adaptive=True, k=k)["children"][:2],
                          POP[:2] & 0xFFFFFFFF)
    assert crossed and kept
    d = rows(2, 1)
    d[0, :3] = (0.01, 0.1, 1.0)
    d[0, 3] = 0.29                               # mutp k4 = 0.3
    assert int(breed(POP, fit, d, cross_rate=0.0, mut_rate=0.0, adaptive=True, k=k)["children"][0, 0]) != 0x0F0F0F0F
    d[0, 3] = 0.31
    assert int(breed(POP, fit, d, cross_rate=0.0, mut_rate=0.0, adaptive=True, k=k)["children"][0, 0]) == 0x0F0F0F0F


def test_device_adapt_prob_at_max():
    fit = [100.0, 60.0, 40.0, 0.0]               # max 100, mean 50; the better parent at the max
    d = rows(2, 1)
    d[0, :3] = (0.1, 0.7, 0.0)                   # r = 20 -> 0, r = 140 -> 1; crossp 0: no crossover
    # (mutp is 1 * (100 - 60) / 50 = 0.8: the bit draws stay at 0.99)
    r = breed(POP[:4], fit, d, cross_rate=0.0, mut_rate=0.0, adaptive=True, k=(1.0, 1.0, 0.5, 0.5))
    np.testing.assert_array_equal(r["children"][:2], POP[:2] & 0xFFFFFFFF)


# --- crossover (tests/test_gaboom.cpp:461-497) ----------------------------------------------------

@pytest.mark.parametrize("intragenes", [False, True])
def test_device_crossover_conserves_material(intragenes):
    ng = 2
    pop = np.array([[0x0F0F0F0F, 0x00FF00FF], [0xF0F0F0F0, 0xFF00FF00]], np.int64)
    n = 500
    d = np.random.default_rng(42).random((n, evaluator.ga_draws_per_pair(ng)))
    d[:, 0], d[:, 1] = 0.25, 0.75                # parents 0 and 1 (equal fitness)
    r = breed(pop, [1.0, 1.0], d, cross_rate=1.0, mut_rate=0.0, intragenes=intragenes)
    ch = r["children"].reshape(n, 2, ng)
    for j, m in ch:
        assert np.all((j | m) == (pop[0] | pop[1]))
        assert np.all((j & m) == (pop[0] & pop[1]))
    # and bit for bit what the restated operator does with the same draws
    f = ga.Fitness.given([1.0, 1.0])
    for k in range(n):
        it = iter(d[k])
        want = ga.pair_with(pop, f, lambda: next(it), 1.0, 0.0, intragenes)
        np.testing.assert_array_equal(ch[k], np.array(want))


def test_device_crossover_single_gene_symmetric():
    pop = np.array([[0xAAAAAAAA], [0x55555555]], np.int64)
    n = 500
    d = np.random.default_rng(123).random((n, evaluator.ga_draws_per_pair(1)))
    d[:, 0], d[:, 1] = 0.25, 0.75
    ch = breed(pop, [1.0, 1.0], d, cross_rate=1.0, mut_rate=0.0, intragenes=True)["children"].reshape(n, 2)
    jc, mc = ch[:, 0] != 0xAAAAAAAA, ch[:, 1] != 0x55555555
    np.testing.assert_array_equal(jc, mc)
    assert jc.sum() > 400


# --- mutate (tests/test_gaboom.cpp:499-523) -------------------------------------------------------

def test_device_mutate_zero_and_full_rate():
    pop = np.array([[0x12345678, 0xABCDEF01, 0x0]], np.int64)
    d = np.random.default_rng(1).random((1, evaluator.ga_draws_per_pair(3)))
    d[0, 2] = 1.0                                # no crossover
    r0 = breed(pop, [1.0], d, cross_rate=0.0, mut_rate=0.0)
    np.testing.assert_array_equal(r0["children"][0], pop[0])
    zero = np.zeros((1, 1), np.int64)
    d1 = np.random.default_rng(2).random((1, evaluator.ga_draws_per_pair(1)))
    d1[0, 2] = 1.0
    r1 = breed(zero, [1.0], d1, cross_rate=0.0, mut_rate=1.0)
    assert int(r1["children"][0, 0]) == 0xFFFFFFFF and int(r1["children"][1, 0]) == 0xFFFFFFFF


# --- roulette_wheel (tests/test_gaboom.cpp:525-564) ----------------------------------------------

def parents_chosen(fitness, u):
    """Breeds one pair per draw u (both roulette draws = u, no crossover, no mutation); the child
    genes name the parent (population entry i holds gene value i)."""
    P = len(fitness)
    pop = np.arange(P, dtype=np.int64).reshape(P, 1)
    d = rows(1, len(u))
    d[:, 0] = u
    d[:, 1] = u
    d[:, 2] = 1.0
    return breed(pop, fitness, d, cross_rate=0.0, mut_rate=0.0)["children"][0::2, 0]


def test_device_roulette():
    u = np.random.default_rng(42).random(100)
    sel = parents_chosen([1.0] * 5, u[:50])
    assert np.all((sel >= 0) & (sel < 5))
    assert (parents_chosen([0.001, 0.001, 1000.0], u) == 2).sum() > 90
    assert parents_chosen([5.0], [0.7])[0] == 0
    np.testing.assert_array_equal(parents_chosen([1.0, 2.0, 3.0], [0.0, 1.0 / 6.0, 0.5, 0.999]), [0, 1, 2, 2])


# --- calc_rmsp through the niche counts (tests/test_gaboom.cpp:566-590) ---------------------------

def test_device_niche_counts_known_distances():
    np.testing.assert_array_equal(evaluator.ga_niche_counts([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0]], 2.0), [1.5, 1.5])
    np.testing.assert_array_equal(evaluator.ga_niche_counts([[1.0, 2.0, 3.0], [1.0, 2.0, 3.0]], 2.0), [2.0, 2.0])
    s = evaluator.ga_niche_counts([[3.0, 4.0], [0.0, 0.0]], 10.0)
    assert s[0] == s[1]
    # the kernel contracts the squared differences into fused multiply-adds; the reference sums them
    # with Eigen's vectorised squaredNorm, in yet another order: agreement to rounding
    rng = np.random.default_rng(5)
    ic = rng.normal(size=(300, 7)) * 3.0
    np.testing.assert_allclose(evaluator.ga_niche_counts(ic, 4.0, 1.0), ga.niche_counts(ic, 4.0, 1.0), rtol=1e-12)
    np.testing.assert_allclose(evaluator.ga_niche_counts(ic, 4.0, 2.0), ga.niche_counts(ic, 4.0, 2.0), rtol=1e-12)


# --- the whole pair on random draws, against the restatement ------------------------------------

@pytest.mark.parametrize("intragenes,adaptive", [(False, False), (True, False), (False, True), (True, True)])
def test_device_pairs_equal_restatement(intragenes, adaptive):
    rng = np.random.default_rng(7 + 2 * intragenes + adaptive)
    P, ng, n = 40, 9, 300
    pop = rng.integers(0, 2 ** 32, size=(P, ng), dtype=np.int64)
    fit = rng.random(P) * 10.0
    order = rng.permutation(P).astype(np.int32)
    prob = [-1.0] * (ng - 2) + [0.3, 0.05]
    k = (1.0, 0.5, 1.0, 0.5)
    d = rng.random((n, evaluator.ga_draws_per_pair(ng)))
    r = breed(pop, fit, d, cross_rate=0.8, mut_rate=0.02, order=order, gene_prob=prob,
              intragenes=intragenes, adaptive=adaptive, k=k)
    f = ga.Fitness.given(fit, order)
    ch = r["children"].reshape(n, 2, ng)
    for kk in range(n):
        pos = [0]

        def draw():
            v = d[kk, pos[0]]
            pos[0] += 1
            return v

        want = ga.pair_with(pop, f, draw, 0.8, 0.02, intragenes, adaptive, k,
                            [float(np.float32(x)) if x >= 0 else -1.0 for x in prob])
        np.testing.assert_array_equal(ch[kk], np.array(want))
        assert r["draws_used"][kk] == pos[0]
