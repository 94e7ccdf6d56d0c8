"""The device GA engine: a generation equals the restated operators on the same draws, a job's
result is the same alone and among other jobs, and the best energy never rises."""
import numpy as np
import pytest

from flexaidds_gb300 import evaluator, prepare, synth, system
from oracle import ga as ref_ga
from oracle import port

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def systems():
    base = system.make_inputs(1200, 7.0, 14, 4, seed=91)
    out = [prepare.prepare(base)]
    for k, (n, t) in enumerate([(20, 6), (10, 2)]):
        lig = synth.random_ligand(n, t, seed=300 + k)
        out.append(prepare.prepare(system.SystemInputs(receptor=base.receptor, ligand=lig,
                                                       grid_xyz=base.grid_xyz, emat=base.emat)))
    return out


# (precision, mutation rate, options): the reference's defaults, then its other operators; the
# low mutation rate makes children that repeat a chromosome the job has made (dropped unless
# duplicates are allowed)
GA_CASES = [
    (0, 0.02, dict()),
    (1, 0.02, dict(intragenes=True, adaptive=True, n_new=58)),
    (0, 0.02, dict(steady=True, n_new=20, adaptive=True, k=(0.8, 0.3, 0.9, 0.2))),
    (0, 0.001, dict(fitness="LINEAR")),
    (1, 0.001, dict(duplicates=True, n_new=31, fitness="SMFREE", entropy_weight=0.3,
                    temperature=500.0, adaptive=True)),
    (0, 0.02, dict(sharing_alpha=2.0, sharing_peaks=3.0, sharing_scale=4.0, adaptive=True)),
    (0, 0.02, dict(steady=True, n_new=40, fitness="SMFREE")),
]
FITNESS_KEYS = ("sharing_alpha", "sharing_peaks", "sharing_scale", "entropy_weight", "temperature")


@pytest.mark.parametrize("prec,pm,opts", GA_CASES)
def test_generation_matches_restated_operators(systems, prec, pm, opts):
    d = systems[0]
    P, seed, pc = 96, 12345, 0.9
    ev = evaluator.GPUEvaluator(d, max_poses=P, precision=prec)
    check = evaluator.GPUEvaluator(d, max_poses=P, precision=prec)
    eng = evaluator.GAEngine(max_jobs=2, precision=prec)
    slot = eng.admit(eng.job(ev, P, 3, seed, pc, pm, **opts), ev)
    rej = ref_ga.Rejector(d, allow=opts.get("duplicates", False))
    # generation 0: the uniform draws, evaluated and sorted
    init = ref_ga.initial_genes(seed, P, d.n_genes, rej)
    e0 = check.eval_genes(init)["evalue"]
    want_g, want_e = ref_ga.boom(init[:0], e0[:0], init, e0)
    pop, pe = eng.read_population(slot, P)
    np.testing.assert_array_equal(pop, want_g)
    np.testing.assert_array_equal(pe, want_e)
    snaps = []
    bopts = {k: v for k, v in opts.items() if k in ("intragenes", "adaptive", "k")}
    fopts = {k.replace("sharing_", ""): v for k, v in opts.items() if k in FITNESS_KEYS}
    nnew = opts.get("n_new", 0)
    for gen in range(3):
        fz = ref_ga.Fitness(pop, pe, d, opts.get("fitness", "PSHARE"), initial=gen == 0, **fopts)
        child = ref_ga.breed(pop, gen, seed, pc, pm, nnew=nnew, rej=rej, fitness=fz, **bopts)
        ce = check.eval_genes(child)["evalue"]
        if opts.get("steady"):
            want_g, want_e = ref_ga.steady(pop, pe, child, ce)
        else:
            want_g, want_e = ref_ga.boom(pop, pe, child, ce)
        eng.step()
        pop, pe = eng.read_population(slot, P)
        np.testing.assert_array_equal(pop, want_g)
        np.testing.assert_array_equal(pe, want_e)
        snaps.append((want_g, want_e))
        assert eng.duplicates(slot) == (rej.rejected, 0)
    if pm < 0.01 and not opts.get("duplicates"):
        assert rej.rejected > 0, "the case was meant to make duplicates"
    assert eng.finished() == [slot]
    # the statmech ensemble: snapshots sorted, near-duplicates removed
    kept = ref_ga.ensemble(snaps, d)
    g, e, th = eng.collect(slot, 300.0)
    assert th["n_ensemble"] == len(kept)
    want = port.thermo(kept, None, 300.0)
    for k in ("log_Z", "free_energy", "mean_energy", "entropy"):
        assert abs(th[k] - want[k]) <= 1e-9 * max(1.0, abs(want[k])), k
    # Cv = (<E^2> - <E>^2) / (kT)^2 cancels: its rounding scales with <E^2> / (kT)^2, not with Cv
    kT = 0.001987206 * 300.0
    assert abs(th["heat_capacity"] - want["heat_capacity"]) <= 1e-9 * max(1.0, want["mean_energy_sq"] / kT ** 2)


def test_job_alone_equals_job_in_a_mix(systems):
    jobs = [(0, 128, 6, 7), (1, 200, 4, 8), (2, 64, 9, 9)]

    def run(which, stagger):
        eng = evaluator.GAEngine(max_jobs=4)
        evs = {k: evaluator.GPUEvaluator(systems[k], max_poses=256) for k, *_ in jobs}
        slots, results = {}, {}
        pending = [j for j in jobs if j[0] in which]
        step = 0
        while pending or eng.jobs:
            # admit one waiting job every `stagger` generations (continuous batching)
            if pending and step % stagger == 0:
                k, P, G, seed = pending.pop(0)
                slots[eng.admit(eng.job(evs[k], P, G, seed), evs[k])] = k
            eng.step()
            step += 1
            for s in eng.finished():
                results[slots[s]] = eng.collect(s, 300.0)
        return results

    mixed = run({0, 1, 2}, 2)
    for k in (0, 1, 2):
        alone = run({k}, 1)[k]
        g, e, th = mixed[k]
        np.testing.assert_array_equal(g, alone[0])
        assert e == alone[1]
        for key in th:
            assert th[key] == alone[2][key] or abs(th[key] - alone[2][key]) <= 1e-12 * abs(alone[2][key])


def test_best_energy_never_rises(systems):
    d = systems[1]
    P = 256
    ev = evaluator.GPUEvaluator(d, max_poses=P)
    eng = evaluator.GAEngine(max_jobs=1)
    slot = eng.admit(eng.job(ev, P, 12, 4242), ev)
    best = [eng.read_population(slot, P)[1][0]]
    for _ in range(12):
        eng.step()
        best.append(eng.read_population(slot, P)[1][0])
    assert all(b <= a for a, b in zip(best, best[1:]))
    assert best[-1] < best[0]
    g, e, th = eng.collect(slot, 300.0)
    assert e == best[-1]
    assert np.isfinite(th["free_energy"])
    launches, graphs = eng.take_launches()
    assert graphs == 12 and launches == 10 + 12 * 10


def test_duplicates_let_through_when_no_new_chromosome_exists(systems):
    """With crossover and mutation off every child repeats a parent: the reference would loop
    for new chromosomes forever; the engine takes them as they come after 16 batches, counts
    them, and the run completes with the population unchanged."""
    d = systems[2]
    P = 8
    ev = evaluator.GPUEvaluator(d, max_poses=P)
    eng = evaluator.GAEngine(max_jobs=1)
    slot = eng.admit(eng.job(ev, P, 2, 99, cross_rate=0.0, mut_rate=0.0, fitness="LINEAR"), ev)
    g0, e0 = eng.read_population(slot, P)
    for _ in range(2):
        eng.step()
    assert eng.finished() == [slot]
    rejected, forced = eng.duplicates(slot)
    assert forced == 2 * P and rejected > 0
    g2, e2 = eng.read_population(slot, P)
    assert set(map(tuple, g2.tolist())) <= set(map(tuple, g0.tolist()))
    assert e2[0] == e0[0]
    eng.collect(slot, 300.0)
