"""Restatement of one GA generation for checking the device GA engine.

TEST INFRASTRUCTURE ONLY: the checker for flexaidds_gb300/csrc/fxe_ga.cu, used by tests/.

Operators as the reference defines them — LINEAR, PSHARE and SMFREE fitness
(LIB/gaboom.cpp:1627-1760) with the roulette order PSHARE implies (:498-499), roulette selection
(:1158-1186), the reproduce loop's crossover-then-mutate of each pair (:918-960), the
bit crossover with intragenes (:2517-2614) and bit mutation (:2620-2641), duplicate rejection by
hash_genes signature (:977-1018, 1040-1045, and the populate loop :1936-1978), BOOM replacement
(:1023-1033) — driven by the counter-based draws the device uses (the reference's own draws come
from a random_device-seeded generator and cannot be replayed).

Not restated: the device lets duplicates through after 16 batches of candidates in a row without
enough new ones (the reference loops on); the tests check that this never happened.
"""
from __future__ import annotations

import math

import numpy as np

M64 = (1 << 64) - 1


def mix64(z: int) -> int:
    """SplitMix64 finaliser (Steele, Lea and Flood, OOPSLA 2014)."""
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def uniform(seed: int, stream: int, k: int) -> float:
    return (mix64(seed ^ mix64((stream * 0x100000001B3 + k) & M64)) >> 11) * 2.0 ** -53


def signature(ic_row) -> int:
    """hash_genes (LIB/gaboom.cpp:1040-1045) of one chromosome's decoded ICs; std::hash<int32_t>
    is the identity, sign-extended to 64 bits."""
    h = 0
    for v in ic_row:
        x = int(float(v) + 0.5) & M64          # (int32_t)(to_ic + 0.5): truncation toward zero
        h ^= (x + 0x9E3779B9 + ((h << 6) & M64) + (h >> 2)) & M64
    return h


class Rejector:
    """The set of signatures a job has produced (duplicates = false): `take` says whether a
    chromosome is new, and remembers it."""

    def __init__(self, desc, allow: bool = False):
        self.desc, self.allow, self.seen, self.rejected = desc, allow, set(), 0

    def take(self, genes) -> bool:
        if self.allow:
            return True
        sig = signature(self.desc.genes_to_ic(np.asarray(genes, np.uint32).astype(np.int32)[None])[0])
        if sig in self.seen:
            self.rejected += 1
            return False
        self.seen.add(sig)
        return True


def gene_probs(desc) -> list:
    """Per gene: the side chain's probability for a rotamer gene (flxsc.prob), else -1."""
    return [float(np.float32(desc.flex_prob[int(desc.gene_atm[g])])) if int(desc.gene_typ[g]) == 4 else -1.0
            for g in range(desc.n_genes)]


INIT_ROT_STREAM = 0xFFFFFFFE


def initial_genes(seed: int, P: int, ng: int, rej: Rejector | None = None, prob=None) -> np.ndarray:
    """Uniform chromosomes; candidate c's gene q is draw c * ng + q. A rotamer gene (prob[q] >= 0)
    is drawn only with its side chain's probability, else 0 (generate_random_individual,
    LIB/gaboom.cpp:1875-1895). With `rej`, candidates whose signature was seen are skipped (the
    populate loop)."""
    prob = prob or [-1.0] * ng
    out, c = [], 0
    while len(out) < P:
        g = []
        for q in range(ng):
            i = c * ng + q
            take = prob[q] < 0 or uniform(seed, INIT_ROT_STREAM, i) < prob[q]
            g.append(mix64(seed ^ mix64((0xFFFFFFFF * 977 + i) & M64)) >> 33 if take else 0)
        c += 1
        if rej is None or rej.take(g):
            out.append(g)
    return np.asarray(out, np.int64).astype(np.int32).reshape(P, ng)


KB = 0.001987206   # kcal/mol/K, LIB/statmech.h:26


def sig_share(desc, peaks: float = 5.0, scale: float = 10.0) -> float:
    """GB->sig_share from the gene limits (LIB/gaboom.cpp:300-309)."""
    ng = desc.n_genes
    s = 0.0
    for g in range(ng):
        w = float(desc.gene_max[g]) - float(desc.gene_min[g])
        s += w * w
    return math.sqrt(s / ng) / (2.0 * math.pow(peaks, 1.0 / ng)) / scale


def calc_rmsp(ic1, ic2) -> float:
    """calc_rmsp (LIB/gaboom.cpp:2874-2885): root mean square of the IC differences, the squares
    summed in gene order."""
    acc = 0.0
    for a, b in zip(ic1, ic2):
        d = float(a) - float(b)
        acc += d * d
    return math.sqrt(acc / len(ic1))


def fitness_stats(fit) -> tuple:
    """fitness_stats (LIB/gaboom.cpp:818-840) over fitness values in roulette order: (running
    sums, total, maximum, mean)."""
    cum, mx, tot = [], float(fit[0]), 0.0
    for f in fit:
        tot += float(f)
        cum.append(tot)
        mx = max(mx, float(f))
    return cum, tot, mx, tot / len(fit)


def adapt_prob(fit_max: float, fit_avg: float, f1: float, f2: float, k) -> tuple:
    """adapt_prob (LIB/gaboom.cpp:848-880): (crossover, mutation) probabilities of a pair whose
    fitness is f1, f2; k = (k1, k2, k3, k4). The denominator is floored at 1e-15
    (GA_FITNESS_DENOM_FLOOR, LIB/ga_constants.h:38)."""
    hi, lo = max(f1, f2), min(f1, f2)
    denom = max(fit_max - fit_avg, 1e-15)
    crossp = k[0] * (fit_max - hi) / denom if hi > fit_avg else k[2]
    mutp = k[1] * (fit_max - lo) / denom if lo > fit_avg else k[3]
    return crossp, mutp


def remove_dups(ic, tol: float = 0.1) -> list:
    """remove_dups (LIB/gaboom.cpp:2728-2747) over chromosomes in their given order: a
    chromosome is dropped when every gene is within tol of the last one kept. Returns the kept
    indices."""
    kept, last = [], None
    for i, row in enumerate(ic):
        if last is None or not all(abs(float(a) - float(b)) < tol for a, b in zip(row, last)):
            kept.append(i)
            last = row
    return kept


def clamped_ic(desc, genes) -> np.ndarray:
    """to_ic of evaluated chromosomes: decoded, then clamped by eval_chromosome
    (LIB/gaboom.cpp:1851-1859)."""
    return np.clip(desc.genes_to_ic(genes), desc.gene_min, desc.gene_max)


class Fitness:
    """calculate_fitness (LIB/gaboom.cpp:1627-1760) of a population sorted by energy, the order
    roulette_wheel walks it in (energy order; fitness order, descending, after a generation under
    PSHARE, LIB/gaboom.cpp:498-499), its running sums and fitness_stats (:818-840). Niche counts
    sum the reference's share term in order over j, the rmsp sum in order over the genes (the
    reference's Eigen reduction may round its last bit otherwise); SMFREE's Boltzmann term is
    exp(-beta (E_i - E_min)), the weight over the largest weight."""

    def __init__(self, pop, pop_e, desc, model="PSHARE", initial=False, alpha=1.0, peaks=5.0,
                 scale=10.0, entropy_weight=0.5, temperature=300.0):
        P = len(pop)
        fit = [float(P - i) for i in range(P)]
        rank_only = model == "LINEAR" or (model == "SMFREE" and not temperature > 0)
        if not rank_only:
            ic = clamped_ic(desc, pop)
            ng = ic.shape[1]
            sig = sig_share(desc, peaks, scale)
            share = niche_counts(ic, sig, alpha)
            if model == "PSHARE":
                fit = [fit[i] / share[i] for i in range(P)]
            else:
                beta = 1.0 / (KB * temperature)
                e = [float(x) for x in pop_e]
                e0 = e[0] if math.isfinite(e[0]) else 0.0
                out = []
                for i in range(P):
                    bw = math.exp(-beta * (e[i] - e0)) if (math.isfinite(e[i]) and math.isfinite(e[0])) else 0.0
                    blended = (1.0 - entropy_weight) * (fit[i] / P) + entropy_weight * bw
                    out.append(blended * P / share[i])
                fit = out
        order = list(range(P))
        if model == "PSHARE" and not initial:
            order = sorted(range(P), key=lambda i: (-fit[i], i))
        self.order = order
        self.fit = [fit[i] for i in order]
        self.cum, self.total, self.max, self.avg = fitness_stats(self.fit)

    @classmethod
    def given(cls, fit, order=None) -> "Fitness":
        """Fitness values given in roulette order (population positions `order`, default
        0..P-1)."""
        self = cls.__new__(cls)
        self.fit = [float(f) for f in fit]
        self.order = list(order) if order is not None else list(range(len(self.fit)))
        self.cum, self.total, self.max, self.avg = fitness_stats(self.fit)
        return self

    def roulette(self, u: float) -> int:
        """roulette_wheel (LIB/gaboom.cpp:1158-1186): a roulette position."""
        return roulette(self.cum, self.total, u)


def niche_counts(ic, sig: float, alpha: float) -> list:
    """PSHARE's niche count of each chromosome (LIB/gaboom.cpp:1652-1661): the sum over all j, in
    order, of 1 - (rmsp / sig_share)^alpha for every rmsp within sig_share."""
    P = len(ic)
    share = []
    for i in range(P):
        s = 0.0
        for j in range(P):
            r = calc_rmsp(ic[i], ic[j])
            if r <= sig:
                s += 1.0 - (r / sig if alpha == 1.0 else math.pow(r / sig, alpha))
        share.append(s)
    return share


def roulette(cum, total: float, u: float) -> int:
    """roulette_wheel (LIB/gaboom.cpp:1158-1186) over running fitness sums: the first position
    whose running sum exceeds u * total, the last if none does, a uniform position when the total
    is not positive."""
    P = len(cum)
    if not total > 0.0:
        return int(u * P) % P
    r = u * total
    for k, c in enumerate(cum):
        if c > r:
            return k
    return P - 1


def roulette_linear(P: int, u: float) -> int:
    tot = float(P) * float(P + 1) * 0.5
    r = u * tot
    lo, hi = 0, P - 1
    while lo < hi:
        mid = (lo + hi) >> 1
        cum = float(mid + 1) * P - 0.5 * float(mid) * float(mid + 1)
        if cum > r:
            hi = mid
        else:
            lo = mid + 1
    return lo


def _mask(np_: int) -> int:
    return 0xFFFFFFFF if np_ >= 31 else (2 << np_) - 1


def breed(pop: np.ndarray, gen: int, seed: int, cross_rate: float, mut_rate: float, nnew: int = 0,
          intragenes: bool = False, adaptive: bool = False, k=(1.0, 0.5, 1.0, 0.5),
          rej: Rejector | None = None, fitness: Fitness | None = None, prob=None) -> np.ndarray:
    """nnew children of generation gen + 1 from the energy-sorted population `pop` (P, ng) int32
    with its `fitness` (LINEAR when None): pair kk's child 1, then its child 2, each kept unless
    `rej` has seen it, until there are nnew."""
    P, ng = pop.shape
    nnew = nnew or P
    out = []
    kk = 0
    while len(out) < nnew:
        for ch in pair(pop, gen, seed, kk, cross_rate, mut_rate, intragenes, adaptive, k, fitness, prob):
            if rej is None or rej.take(ch):
                out.append(ch)
                if len(out) == nnew:
                    break
        kk += 1
    return np.asarray(out, np.int64).astype(np.uint32).astype(np.int32)


def pair(pop: np.ndarray, gen: int, seed: int, kk: int, cross_rate: float, mut_rate: float,
         intragenes: bool, adaptive: bool, k, fitness: Fitness | None = None, prob=None):
    """Pair kk of generation gen + 1's children (two lists of uint32 genes)."""
    P = pop.shape[0]
    if fitness is None:
        fitness = Fitness(pop, np.zeros(P), None, "LINEAR")
    st = ((gen + 1) << 32) + kk
    d = 0

    def draw():
        nonlocal d
        v = uniform(seed, st, d)
        d += 1
        return v

    return pair_with(pop, fitness, draw, cross_rate, mut_rate, intragenes, adaptive, k, prob)


def pair_with(pop: np.ndarray, fitness: Fitness, draw, cross_rate: float, mut_rate: float,
              intragenes: bool = False, adaptive: bool = False, k=(1.0, 0.5, 1.0, 0.5), prob=None):
    """One pair of children from the draws draw() hands out, in the reference's order: two
    roulette draws, adapt_prob when adaptive, the crossover draw and the crossover's own, then
    each child's mutation draws (the reproduce loop, LIB/gaboom.cpp:918-964)."""
    ng = pop.shape[1]
    u32 = pop.astype(np.int64) & 0xFFFFFFFF
    pa = fitness.roulette(draw())
    pb = fitness.roulette(draw())
    a, b = fitness.order[pa], fitness.order[pb]
    crossp, mutp = cross_rate, mut_rate
    if adaptive:
        crossp, mutp = adapt_prob(fitness.max, fitness.avg, fitness.fit[pa], fitness.fit[pb], k)
    john = [int(x) for x in u32[a]]
    mary = [int(x) for x in u32[b]]
    if draw() < crossp:
        crossover(john, mary, intragenes, draw)
    for ch in (john, mary):
        mutate(ch, mutp, draw, prob or [-1.0] * ng)
    return john, mary


def crossover(john: list, mary: list, intragenes: bool, draw) -> None:
    """crossover (LIB/gaboom.cpp:2517-2614) of two chromosomes' uint32 genes in place: two gene
    draws, then two bit points (inside genes) or two gene-boundary choices, bits swapped between
    the points. draw() gives the next uniform in [0, 1)."""
    ng = len(john)
    gen_a = min(int(draw() * ng), ng - 1)
    gen_b = min(int(draw() * ng), ng - 1)
    if intragenes:
        pnt_a = int(draw() * 32.0)
        pnt_b = int(draw() * 32.0)
        if gen_a > gen_b:
            gen_a, gen_b, pnt_a, pnt_b = gen_b, gen_a, pnt_b, pnt_a
        if gen_a == gen_b and pnt_a < pnt_b:
            pnt_a, pnt_b = pnt_b, pnt_a
    else:
        if gen_a > gen_b:
            gen_a, gen_b = gen_b, gen_a
        if gen_a != gen_b:
            pnt_a = 32 if draw() < 0.5 else 0
            pnt_b = 32 if draw() < 0.5 else 0
            if gen_b - gen_a == 1 and pnt_a == 0 and pnt_b == 32:
                pnt_b = pnt_a
        else:
            pnt_a, pnt_b = 32, 0
    for j in range(gen_a, gen_b + 1):
        m = _mask(pnt_a if j == gen_a else 32)
        uj, um = john[j], mary[j]
        john[j] = (uj & ~m & 0xFFFFFFFF) | (um & m)
        mary[j] = (uj & m) | (um & ~m & 0xFFFFFFFF)
    if pnt_b > 0:
        m = _mask(pnt_b - 1)
        uj, um = john[gen_b], mary[gen_b]
        john[gen_b] = (uj & ~m & 0xFFFFFFFF) | (um & m)
        mary[gen_b] = (uj & m) | (um & ~m & 0xFFFFFFFF)


def mutate(ch: list, mutp: float, draw, prob=None) -> None:
    """mutate (LIB/gaboom.cpp:2620-2641) of one chromosome's uint32 genes in place: each bit
    flipped when its draw falls under mutp; a rotamer gene (prob[q] >= 0) only when a first draw
    falls under its side chain's probability (LIB/gaboom.cpp:944-966)."""
    prob = prob or [-1.0] * len(ch)
    for q in range(len(ch)):
        if prob[q] >= 0 and not draw() < prob[q]:
            continue
        m = 0
        for bit in range(32):
            if draw() < mutp:
                m |= 1 << bit
        ch[q] ^= m


def steady(pop: np.ndarray, pop_e: np.ndarray, child: np.ndarray, child_e: np.ndarray):
    """STEADY replacement: child i in the place of parent P-1-i, then sorted by energy (then by
    place)."""
    P, nnew = pop.shape[0], child.shape[0]
    genes = pop.copy()
    e = pop_e.astype(np.float64).copy()
    for i in range(nnew):
        genes[P - 1 - i] = child[i]
        e[P - 1 - i] = child_e[i]
    e = np.where(np.isnan(e), np.inf, e)
    order = np.lexsort((np.arange(P), e))
    return genes[order], e[order]


def boom(pop: np.ndarray, pop_e: np.ndarray, child: np.ndarray, child_e: np.ndarray):
    """Parents and children merged, sorted by energy (then by position), the best P kept (the
    initial population, which has no parents: all of it)."""
    keep = pop.shape[0] if pop.shape[0] else child.shape[0]
    e = np.concatenate([pop_e, child_e]).astype(np.float64)
    e = np.where(np.isnan(e), np.inf, e)
    order = np.lexsort((np.arange(e.shape[0]), e))[:keep]
    genes = np.concatenate([pop, child])[order]
    return genes, e[order]


def ensemble(snapshots, desc) -> np.ndarray:
    """The reference's statmech ensemble (LIB/gaboom.cpp:494,520-540,2728-2747): every
    generation's population, sorted by energy (ties in snapshot order), a chromosome dropped
    when every decoded gene is within 0.1 of the last one kept. Returns the kept energies."""
    g = np.concatenate([s[0] for s in snapshots])
    e = np.concatenate([s[1] for s in snapshots])
    ic = clamped_ic(desc, g)
    order = np.argsort(e, kind="stable")
    return np.asarray(e[order][remove_dups(ic[order])])
