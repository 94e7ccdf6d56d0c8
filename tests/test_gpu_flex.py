"""Flexible side chains on the CUDA path, against the oracle through the C ABI.

The oracle's side chains are pinned to the compiled reference by the flex_* golden fixtures
(tests/test_oracle.py, tests/test_gpu_parity.py::test_golden_fixtures); here the CUDA path is
checked against the oracle on larger seeded sets: every status class, the complementarity terms
of every scored pose, the contact lists of side-chain and ligand atoms, the rotamer selected by
the gene value, and the side chains' place in batched launches and in the GA engine.
"""
import numpy as np
import pytest

from flexaidds_gb300 import evaluator, prepare, synth, system
from oracle import ga as ref_ga
from oracle import port

pytestmark = pytest.mark.gpu

REF, FAST = evaluator.GPUEvaluator.REFERENCE, evaluator.GPUEvaluator.FAST


def rel_err(a, b):
    return np.abs(a - b) / np.maximum(1.0, np.abs(b))


def oracle_eval(d, ic, **kw):
    port.set_reference_compat(True)
    port.set_trig_rounding(False)
    return port.Oracle(d).eval_ic(ic, **kw)


def enriched(d, n_pool, seed, scored, other):
    pool = synth.random_genes(n_pool, d.n_genes, seed=seed)
    st = oracle_eval(d, d.genes_to_ic(pool))["cf"]["status"]
    sel = np.concatenate([np.nonzero(st == 0)[0][:scored], np.nonzero(st != 0)[0][:other]])
    return pool[np.sort(sel)]


@pytest.fixture(scope="module")
def flex():
    d = prepare.prepare(system.make_inputs(2000, 8.0, 24, 6, seed=43, side_chains=3))
    return d, enriched(d, 24000, 44, 400, 200)


@pytest.mark.parametrize("prec", [REF, FAST])
def test_side_chains_against_oracle(flex, prec):
    d, genes = flex
    assert d.n_flex == 3 and d.n_sc > 0
    r = oracle_eval(d, d.genes_to_ic(genes), want_xyz=True)
    ev = evaluator.GPUEvaluator(d, max_poses=1024, precision=prec)
    g = ev.eval_genes(genes)
    np.testing.assert_array_equal(g["status"], r["cf"]["status"])
    ok = g["status"] == 0
    assert ok.sum() >= 250
    rot = d.genes_to_ic(genes)[:, -3:]
    assert len(np.unique(rot[ok])) == 8          # every rotamer among the scored poses
    for p in range(0, len(genes), 7):
        np.testing.assert_array_equal(ev.ligand_xyz(p), r["xyz"][p])
    e = rel_err(g["evalue"], r["cf"]["evalue"])
    assert np.all(e[~ok] <= 1e-6)
    if prec == REF:
        print(f"side chains, reference precision: {ok.sum()} scored, max {e[ok].max():.1e}")
        assert e[ok].max() <= 1e-9
        scale = np.maximum(1.0, np.abs(r["cf"]["evalue"][ok]))
        for k in ("com", "wal", "sas"):
            assert (np.abs(g[k][ok] - r["cf"][k][ok]) / scale).max() <= 1e-9, k
    else:
        bad = (e[ok] > 1e-4).sum()
        print(f"side chains, fast precision: {ok.sum()} scored, median {np.median(e[ok]):.1e}, {bad} beyond 1e-4")
        assert np.median(e[ok]) <= 1e-5
        assert bad <= 0.2 * ok.sum()
    assert ev.stats()["capacity"] == 0
    ev.close()


def test_side_chain_contact_lists(flex):
    d, genes = flex
    genes = genes[:100]
    r = oracle_eval(d, d.genes_to_ic(genes), want_contacts=True)
    ev = evaluator.GPUEvaluator(d, max_poses=128, precision=REF)
    g = ev.eval_genes(genes)
    c = r["contacts"]
    want = {}
    for p, a, q, s in zip(c["pose"], c["atom"], c["partner"], c["area"]):
        want.setdefault((int(p), int(a)), []).append((int(q), float(s)))
    n_side = 0
    for p in np.nonzero(g["status"] == 0)[0]:
        for a in range(d.n_sc + d.n_lig):
            part, area = ev.contacts(int(p), a)
            mine = sorted(zip(part.tolist(), area.tolist()))
            theirs = sorted(want.get((int(p), a), []))
            assert [m[0] for m in mine] == [t[0] for t in theirs], (p, a)
            np.testing.assert_allclose([m[1] for m in mine], [t[1] for t in theirs], rtol=1e-5, atol=1e-5)
            if a < d.n_sc:
                n_side += len(mine)
    assert n_side > 100
    ev.close()


def test_rotamer_gene_rounding(flex):
    """The rotamer is (unsigned)(ic + 0.5) of the clamped gene value (LIB/ic2cf.cpp:90-94)."""
    d, genes = flex
    ic = d.genes_to_ic(genes)
    ok = oracle_eval(d, ic)["cf"]["status"] == 0
    ic = ic[ok][:16].copy()
    vals = np.array([0.0, 0.49, 0.5, 2.49999, 2.5, 6.51, 7.0, 9.0, -3.0])
    for k, v in enumerate(vals):
        ic[k % len(ic), -1 - (k % 3)] = v
    r = oracle_eval(d, ic)["cf"]
    ev = evaluator.GPUEvaluator(d, max_poses=64, precision=REF)
    g = ev.eval_ic(ic)
    np.testing.assert_array_equal(g["status"], r["status"])
    assert rel_err(g["evalue"], r["evalue"]).max() <= 1e-9
    ev.close()


def test_side_chains_with_intramolecular_terms_off():
    inp = system.make_inputs(900, 7.0, 16, 4, seed=45, side_chains=2)
    inp.intramolecular = 0
    d = prepare.prepare(inp)
    genes = enriched(d, 12000, 46, 200, 50)
    r = oracle_eval(d, d.genes_to_ic(genes))["cf"]
    ev = evaluator.GPUEvaluator(d, max_poses=512, precision=REF)
    g = ev.eval_genes(genes)
    np.testing.assert_array_equal(g["status"], r["status"])
    assert (g["status"] == 0).sum() >= 100
    assert rel_err(g["evalue"], r["evalue"]).max() <= 1e-9
    ev.close()


def test_side_chains_in_a_batch(flex):
    """A context with side chains and one without, in one batched launch: records identical to
    one context at a time."""
    d, genes = flex
    d0 = prepare.prepare(system.make_inputs(2000, 8.0, 24, 6, seed=47))
    g0 = synth.random_genes(300, d0.n_genes, seed=48)
    a = evaluator.GPUEvaluator(d, max_poses=1024)
    b = evaluator.GPUEvaluator(d0, max_poses=512)
    alone = [a.eval_genes(genes)["evalue"], b.eval_genes(g0)["evalue"]]
    batch = evaluator.Batch(max_jobs=4, max_poses=2048, max_genes=64)
    out = batch.eval_genes([(a, genes), (b, g0)])
    for k in range(2):
        np.testing.assert_array_equal(out[k]["evalue"], alone[k])
    a.close()
    b.close()


def test_ga_generation_with_side_chains(flex):
    d, _ = flex
    P, seed, pc, pm = 64, 777, 0.9, 0.02
    ev = evaluator.GPUEvaluator(d, max_poses=P)
    check = evaluator.GPUEvaluator(d, max_poses=P)
    eng = evaluator.GAEngine(max_jobs=1)
    slot = eng.admit(eng.job(ev, P, 2, seed, pc, pm), ev)
    rej = ref_ga.Rejector(d)
    prob = ref_ga.gene_probs(d)
    assert sum(p >= 0 for p in prob) == 3
    init = ref_ga.initial_genes(seed, P, d.n_genes, rej, prob)
    assert (init[:, -3:] == 0).any()          # rotamer genes left at rotamer 0 by their chance
    e0 = check.eval_genes(init)["evalue"]
    pop, pe = ref_ga.boom(init[:0], e0[:0], init, e0)
    got = eng.read_population(slot, P)
    np.testing.assert_array_equal(got[0], pop)
    for gen in range(2):
        fz = ref_ga.Fitness(pop, pe, d, "PSHARE", initial=gen == 0)
        child = ref_ga.breed(pop, gen, seed, pc, pm, rej=rej, fitness=fz, prob=prob)
        pop, pe = ref_ga.boom(pop, pe, child, check.eval_genes(child)["evalue"])
        eng.step()
        got = eng.read_population(slot, P)
        np.testing.assert_array_equal(got[0], pop)
        np.testing.assert_array_equal(got[1], pe)
    eng.collect(slot, 300.0)


def test_side_chains_through_the_receptor_cache(flex):
    """A context sharing a receptor with side chains (fxe_context_create_shared) scores another
    ligand exactly as a context with its own copy of the receptor."""
    d, _ = flex
    lig = synth.random_ligand(18, 5, seed=501)
    inp = system.make_inputs(2000, 8.0, 24, 6, seed=43, side_chains=3)
    d2 = prepare.prepare(system.SystemInputs(receptor=inp.receptor, ligand=lig, grid_xyz=inp.grid_xyz,
                                             emat=inp.emat))
    assert d2.n_flex == 3
    genes = enriched(d2, 8000, 502, 150, 50)
    base = evaluator.GPUEvaluator(d, max_poses=8)
    shared = evaluator.GPUEvaluator(d2, max_poses=256, share_receptor_with=base)
    own = evaluator.GPUEvaluator(d2, max_poses=256)
    a, b = shared.eval_genes(genes), own.eval_genes(genes)
    np.testing.assert_array_equal(a["status"], b["status"])
    np.testing.assert_array_equal(a["evalue"], b["evalue"])
    assert (a["status"] == 0).sum() >= 100
    for ev in (shared, own, base):
        ev.close()


def test_side_chains_with_poses_outside_the_box():
    """Anchors beyond the receptor's box: index_protein re-derives the cell grid for those poses,
    and the contact scan bins every rigid atom on it with the side-chain atoms set apart."""
    inp = system.make_inputs(600, 6.0, 10, 2, seed=37, side_chains=2)
    rng = np.random.default_rng(38)
    lo, hi = inp.receptor.xyz.min(axis=0), inp.receptor.xyz.max(axis=0)
    m = 256
    pts = rng.uniform(lo, hi, size=(m, 3))
    axis = rng.integers(0, 3, size=m)
    off = rng.uniform(0.5, 4.0, size=m)
    for k in range(m):
        pts[k, axis[k]] = hi[axis[k]] + off[k] if k % 2 else lo[axis[k]] - off[k]
    inp.grid_xyz = np.ascontiguousarray(np.concatenate([inp.grid_xyz[:256], pts]).astype(np.float32))
    d = prepare.prepare(inp)
    genes = synth.random_genes(3000, d.n_genes, seed=39)
    r = oracle_eval(d, d.genes_to_ic(genes))["cf"]
    ev = evaluator.GPUEvaluator(d, max_poses=3000, precision=REF)
    g = ev.eval_genes(genes)
    np.testing.assert_array_equal(g["status"], r["status"])
    ok = g["status"] == 0
    assert ok.sum() >= 100
    assert rel_err(g["evalue"], r["evalue"]).max() <= 1e-6
    assert rel_err(g["evalue"][ok], r["evalue"][ok]).max() <= 1e-9
    ev.close()
