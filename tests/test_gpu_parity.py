"""CUDA path against the oracle and the reference's golden fixtures, through the C ABI.

Tolerances (per pose, relative to max(1, |E|)):
  * reference precision (FP64 polyhedra, the reference's expressions), identical inputs:
    every scored pose within 1e-9 (observed: median 1e-16, maximum 1e-14, the last-bit
    differences of CUDA's and the C library's atan/acos/sqrt); status classes identical; ligand
    coordinates bit-identical;
  * against the golden fixtures of the compiled reference: every scored pose within 1e-6,
    including the poses whose faces read the slot past their point list (order_faces,
    LIB/Vcontacts.cpp:800-812), which the device replays; status classes identical wherever the
    coordinates are (poses whose coordinates differ in the last bit are counted);
  * fast precision (FP32 polyhedra): median within 1e-5, 1e-4 on most poses; the rest are
    poses where the area formulas are ill-conditioned (counted and printed).

The oracle runs in its reference-compat mode (ptorder cleared before each pose, the stale read
replayed), which reproduces the compiled reference bit for bit.
"""
import numpy as np
import pytest

from flexaidds_gb300 import evaluator, prepare, synth, system
from oracle import port

pytestmark = pytest.mark.gpu

REF, FAST = evaluator.GPUEvaluator.REFERENCE, evaluator.GPUEvaluator.FAST


def rel_err(a, b):
    return np.abs(a - b) / np.maximum(1.0, np.abs(b))


def oracle_eval(d, ic, compat=True, **kw):
    """The oracle with the C library's cosf/sinf in the pose build, as the reference; the CUDA
    build uses the same values, tabulated by the host at context creation. compat: the
    reference's face order (the default of both); False: the geometric one."""
    port.set_reference_compat(compat)
    port.set_trig_rounding(False)
    return port.Oracle(d).eval_ic(ic, **kw)


@pytest.fixture(scope="module")
def c0():
    inp = system.make_inputs(2000, 8.0, 24, 6, seed=41)
    d = prepare.prepare(inp)
    # uniform chromosomes clash nine times in ten: enrich with poses that get scored
    pool = synth.random_genes(24000, d.n_genes, seed=42)
    ic = d.genes_to_ic(pool)
    st = oracle_eval(d, ic)["cf"]["status"]
    sel = np.concatenate([np.nonzero(st == 0)[0][:400], np.nonzero(st != 0)[0][:200]])
    return d, pool[np.sort(sel)]


@pytest.mark.parametrize("prec", [REF, FAST])
def test_random_chromosomes_against_oracle(c0, prec):
    d, genes = c0
    r = oracle_eval(d, d.genes_to_ic(genes), want_xyz=True)
    ev = evaluator.GPUEvaluator(d, max_poses=1024, precision=prec)
    g = ev.eval_genes(genes)
    np.testing.assert_array_equal(g["status"], r["cf"]["status"])
    ok = g["status"] == 0
    assert ok.sum() >= 250
    for p in range(len(genes)):
        np.testing.assert_array_equal(ev.ligand_xyz(p), r["xyz"][p])
    e = rel_err(g["evalue"], r["cf"]["evalue"])
    assert np.all(e[~ok] <= 1e-6)          # sentinels and clash sums
    np.testing.assert_array_equal(g["rclash"][ok], r["cf"]["rclash"][ok])
    if prec == REF:
        print(f"reference precision: {ok.sum()} scored, median {np.median(e[ok]):.1e}, max {e[ok].max():.1e}")
        assert e[ok].max() <= 1e-9, e[ok].max()
        scale = np.maximum(1.0, np.abs(r["cf"]["evalue"][ok]))
        for k in ("com", "wal", "sas"):   # each term, on the scale of the pose's score
            assert (np.abs(g[k][ok] - r["cf"][k][ok]) / scale).max() <= 1e-9, k
    else:
        bad = (e[ok] > 1e-4).sum()
        print(f"fast precision: {ok.sum()} scored, median {np.median(e[ok]):.1e}, {bad} beyond 1e-4")
        assert np.median(e[ok]) <= 1e-5
        assert bad <= 0.2 * ok.sum()
    assert ev.stats()["capacity"] == 0
    ev.close()


def test_geometric_face_order_against_oracle(c0):
    """The geometric face order against the oracle's default mode, which takes the same choice."""
    d, genes = c0
    r = oracle_eval(d, d.genes_to_ic(genes), compat=False)["cf"]
    ev = evaluator.GPUEvaluator(d, max_poses=1024, precision=REF,
                                face_order=evaluator.GPUEvaluator.FACE_ORDER_GEOMETRIC)
    g = ev.eval_genes(genes)
    np.testing.assert_array_equal(g["status"], r["status"])
    ok = g["status"] == 0
    e = rel_err(g["evalue"], r["evalue"])
    assert ok.sum() >= 250
    assert e[ok].max() <= 1e-9, e[ok].max()
    assert ev.stats()["unreplayed_faces"] == 0
    ev.close()


def test_contact_lists_against_oracle(c0):
    d, genes = c0
    genes = genes[:120]
    r = oracle_eval(d, d.genes_to_ic(genes), want_contacts=True)
    ev = evaluator.GPUEvaluator(d, max_poses=256, precision=REF)
    g = ev.eval_genes(genes)
    c = r["contacts"]
    want = {}
    for p, a, q, s in zip(c["pose"], c["atom"], c["partner"], c["area"]):
        want.setdefault((int(p), int(a)), []).append((int(q), float(s)))
    n_checked = 0
    for p in np.nonzero(g["status"] == 0)[0]:
        for a in range(d.n_lig):
            part, area = ev.contacts(int(p), a)
            mine = sorted(zip(part.tolist(), area.tolist()))
            theirs = sorted(want.get((int(p), a), []))
            assert [m[0] for m in mine] == [t[0] for t in theirs], (p, a)
            np.testing.assert_allclose([m[1] for m in mine], [t[1] for t in theirs], rtol=1e-5, atol=1e-5)
            n_checked += len(mine)
    assert n_checked > 300
    ev.close()


def test_golden_fixtures(golden):
    """Against the compiled reference's own results (made by tests/golden/make_golden.py): every
    scored pose within 1e-6, the poses whose faces read the stale slot included."""
    name, d, g = golden
    port.set_reference_compat(False)
    o = port.Oracle(d)
    stale = np.array([o.eval_ic(g["ic"][p:p + 1], counts=True)["counts"]["no_partner"] > 0
                      for p in range(g["ic"].shape[0])])
    ev = evaluator.GPUEvaluator(d, max_poses=512, precision=REF)
    out = ev.eval_genes(g["genes"])
    st = ev.stats()
    same_xyz = np.array([np.array_equal(ev.ligand_xyz(p), g["xyz"][p]) for p in range(len(g["status"]))])
    # the reference moves an atom whose hull walk reaches 200 edges and leaves it there
    # (LIB/Vcontacts.cpp:378-405), so only the coordinates of its failed poses may differ
    assert same_xyz[g["status"] != 1].all()
    np.testing.assert_array_equal(out["status"][same_xyz], g["status"][same_xyz])
    flipped = int((out["status"] != g["status"]).sum())
    assert flipped <= 0.02 * len(same_xyz)
    ok = (g["status"] == 0) & (out["status"] == 0) & same_xyz
    e = rel_err(out["evalue"], g["cf"][:, 9])
    # the same poses with the geometric face order, for the record
    geo = evaluator.GPUEvaluator(d, max_poses=512, precision=REF, face_order=evaluator.GPUEvaluator.FACE_ORDER_GEOMETRIC)
    eg = rel_err(geo.eval_genes(g["genes"])["evalue"], g["cf"][:, 9])
    geo.close()
    print(f"{name}: {ok.sum()} scored ({(ok & stale).sum()} with stale-slot faces, {st['no_partner_faces']} such "
          f"faces, {st['unreplayed_faces']} not replayed); max rel {e[ok].max():.1e} "
          f"(stale-slot poses {e[ok & stale].max() if (ok & stale).any() else 0.0:.1e}); geometric order: "
          f"{(eg[ok] > 1e-4).sum()} beyond 1e-4; {(~same_xyz).sum()} hull failures with moved atoms, "
          f"{flipped} status flips")
    assert st["unreplayed_faces"] == 0
    assert ok.sum() >= 0.9 * ((g["status"] == 0) & same_xyz).sum()
    assert e[ok].max() <= 1e-6
    # clash sums (d^-12) of poses whose coordinates differ in the last bit differ accordingly
    assert np.all(e[(g["status"] != 0) & same_xyz] <= 1e-6)
    ev.close()


def test_scale_system_against_oracle():
    """6,000-atom receptor, 12 A cleft, 48-atom ligand with 12 torsions."""
    inp = system.make_inputs(6000, 12.0, 48, 12, seed=61)
    d = prepare.prepare(inp)
    pool = synth.random_genes(6000, d.n_genes, seed=62)
    ic = d.genes_to_ic(pool)
    r = oracle_eval(d, ic)["cf"]
    sel = np.concatenate([np.nonzero(r["status"] == 0)[0][:150], np.nonzero(r["status"] != 0)[0][:50]])
    ev = evaluator.GPUEvaluator(d, max_poses=256, precision=REF)
    g = ev.eval_genes(pool[sel])
    np.testing.assert_array_equal(g["status"], r["status"][sel])
    ok = g["status"] == 0
    assert ok.sum() >= 20
    assert rel_err(g["evalue"], r["evalue"][sel]).max() <= 1e-9
    ev.close()


def test_uneven_ligand_shape_against_oracle():
    """The batched workloads' largest ligand shape: a 4,000-atom receptor (10 A cleft) and a
    70-atom ligand with 15 torsions. Such a ligand clashes in the cleft for nearly every uniform
    chromosome, so its anchors lie 6-12 A beyond a face of the receptor's box, where a few in a
    hundred poses get scored."""
    base = system.make_inputs(4000, 10.0, 70, 15, seed=91)
    rng = np.random.default_rng(93)
    lo, hi = base.receptor.xyz.min(axis=0), base.receptor.xyz.max(axis=0)
    grid = rng.uniform(lo, hi, size=(400, 3))
    grid[:, 2] = hi[2] + rng.uniform(6.0, 12.0, 400)
    d = prepare.prepare(system.SystemInputs(receptor=base.receptor, ligand=base.ligand,
                                            grid_xyz=grid.astype(np.float32), emat=base.emat))
    pool = synth.random_genes(20000, d.n_genes, seed=92)
    r = oracle_eval(d, d.genes_to_ic(pool))["cf"]
    sel = np.concatenate([np.nonzero(r["status"] == 0)[0][:150], np.nonzero(r["status"] != 0)[0][:50]])
    ev = evaluator.GPUEvaluator(d, max_poses=256, precision=REF)
    g = ev.eval_genes(pool[sel])
    np.testing.assert_array_equal(g["status"], r["status"][sel])
    ok = g["status"] == 0
    e = rel_err(g["evalue"], r["evalue"][sel])
    print(f"70-atom ligand: {ok.sum()} scored of {len(sel)}, max rel {e[ok].max():.1e}, "
          f"{ev.stats()['no_partner_faces']} stale-slot faces replayed")
    assert ok.sum() >= 100
    assert e[ok].max() <= 1e-9
    assert e[~ok].max() <= 1e-6
    assert ev.stats()["capacity"] == 0
    ev.close()


def test_large_ligand_against_oracle():
    """A 120-atom ligand with 15 torsions (the masks and staging hold up to 128 atoms)."""
    base = system.make_inputs(2000, 8.0, 24, 6, seed=41)
    lig = synth.random_ligand(120, 15, seed=77)
    # anchors 4-12 A beyond a face of the receptor's box: the ligand lies against its surface
    rng = np.random.default_rng(79)
    lo, hi = base.receptor.xyz.min(axis=0), base.receptor.xyz.max(axis=0)
    grid = rng.uniform(lo, hi, size=(400, 3))
    grid[:, 0] = hi[0] + rng.uniform(4.0, 12.0, 400)
    d = prepare.prepare(system.SystemInputs(receptor=base.receptor, ligand=lig,
                                            grid_xyz=grid.astype(np.float32), emat=base.emat))
    pool = synth.random_genes(6000, d.n_genes, seed=78)
    r = oracle_eval(d, d.genes_to_ic(pool))["cf"]
    ev = evaluator.GPUEvaluator(d, max_poses=1024, precision=REF)
    g = ev.eval_genes(pool)
    np.testing.assert_array_equal(g["status"], r["status"])
    ok = g["status"] == 0
    e = rel_err(g["evalue"], r["evalue"])
    print(f"120-atom ligand: {ok.sum()} scored of {len(pool)}, max rel {e.max():.1e}")
    assert ok.sum() >= 100
    assert e.max() <= 1e-9
    ev.close()
