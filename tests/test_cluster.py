"""CF-based clustering (cluster, LIB/cluster.cpp:9-218) and the result files.

CPU: the C restatement against the golden fixtures made by the reference's own cluster()
(tests/golden/make_golden_cluster.py: the .cad text it wrote, byte for byte), its invariants, and
the writers' formats (.cad, _par.res). GPU: fxe_cluster through the C ABI against the
restatement on the fixtures and on larger seeded ensembles: heads, frequencies, members and
RMSDs bit for bit, the FP64 TCF/ACF sums within 1e-12 (the device adds them in another order),
and the .cad text identical to the reference's.
"""
import os
import struct

import numpy as np
import pytest

from flexaidds_gb300 import results, synth
from flexaidds_gb300.system import Descriptor
from oracle import port

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CLUSTER_FIXTURES = ("cluster_flex_900_16", "cluster_lig_2000_24")


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = Descriptor.from_arrays(z, "d_")
    cases = [(int(t), float(r), int(m)) for t, r, m in z["cases"]]
    cads = [bytes(z[f"cad_{k}"]).decode() for k in range(len(cases))]
    return d, z["ic"], z["app_evalue"], cases, cads


@pytest.fixture(scope="module", params=CLUSTER_FIXTURES)
def fixture(request):
    return load(request.param)


def oracle_cluster(d, ic, e, T, thr, R):
    port.set_trig_rounding(False)
    return port.Oracle(d).cluster(ic, e, T, thr, R)


def test_oracle_against_reference_cad(fixture):
    d, ic, e, cases, cads = fixture
    for (T, thr, R), cad in zip(cases, cads):
        r = oracle_cluster(d, ic, e, T, thr, R)
        assert results.cad_text(r) == cad, (T, thr, R)


def test_oracle_cluster_invariants(fixture):
    d, ic, e, cases, _ = fixture
    n = ic.shape[0]
    xyz = port.Oracle(d).build_ic(ic).reshape(n, -1)
    for T, thr, R in cases:
        r = oracle_cluster(d, ic, e, T, thr, R)
        nc, mem = r["n_clusters"], r["member_of"]
        heads = np.unique(mem[mem >= 0])
        assert len(heads) == nc <= R
        assert np.all(mem[heads] == heads)
        # a head is the first chromosome of its cluster, and heads come in chromosome order
        for h in heads:
            assert np.nonzero(mem == h)[0][0] == h
        # members are within the threshold of their head (the RMSD recomputed here in float64
        # agrees with the single-precision one to rounding)
        k = np.nonzero(mem >= 0)[0]
        ref = np.sqrt(((xyz[k] - xyz[mem[k]]).astype(np.float64) ** 2).sum(1) / d.n_lig)
        np.testing.assert_allclose(r["rmsd"][k], ref, rtol=1e-5, atol=1e-5)
        assert np.all(r["rmsd"][k] <= thr)
        # frequencies and (at temperature 0) ACF = the cluster's energy sum, in entry order
        real = r["freq"] > 0
        assert r["freq"].sum() == len(k)
        if T == 0:
            for c in range(nc):
                sel = mem == r["top"][c]
                assert r["freq"][c] == sel.sum()
                assert abs(r["acf"][c] - e[sel].sum()) <= 1e-9 * max(1.0, abs(r["acf"][c]))
                assert r["tcf"][c] == e[r["top"][c]]
        else:
            assert np.all(np.diff(r["acf"][: min(R, n)]) >= 0)   # sorted by ACF
            assert real.sum() == nc


def test_unclustered_after_max_results(fixture):
    d, ic, e, _, _ = fixture
    r = oracle_cluster(d, ic, e, 0, 0.5, 3)
    assert r["n_clusters"] == 3
    mem = r["member_of"]
    assert (mem == -1).any()
    assert np.all(r["rmsd"][mem == -1] == 0.0)


def test_cad_text_format():
    res = {"n_clusters": 2, "top": np.array([3, 0, 0]), "freq": np.array([4, 1, 0]),
           "tcf": np.array([-12.5, -3.25, 0.0]), "acf": np.array([-40.0, -3.25, 0.0]),
           "top_rmsd": np.array([[0, 1.5, 0], [1.5, 0, 0], [0, 0, 0]], np.float32)}
    assert results.cad_text(res) == (
        "Cluster 0: TOP=3 TCF=-12.500000 ACF=-40.000000 freq=4\n"
        "Cluster 1: TOP=0 TCF=-3.250000 ACF=-3.250000 freq=1\n"
        "RMSD between clusters\n"
        "rmsd(0,1)=1.500000\n")
    res["n_clusters"] = 1
    assert results.cad_text(res) == "Cluster 0: TOP=3 TCF=-12.500000 ACF=-40.000000 freq=4\n"


def test_par_file_layout(tiny_system):
    """write_par (LIB/gaboom.cpp:2771-2803): "genes", one 48-byte genlim per gene, "chrom", the
    int32 genes chromosome by chromosome."""
    _, d = tiny_system
    genes = synth.random_genes(7, d.n_genes, seed=3)
    data = results.par_bytes(d, genes)
    ng = d.n_genes
    assert len(data) == 5 + 48 * ng + 5 + 4 * 7 * ng
    assert data[:5] == b"genes" and data[5 + 48 * ng:10 + 48 * ng] == b"chrom"
    lim, back = results.read_par(data, ng)
    np.testing.assert_array_equal(back, genes)
    for g in range(ng):
        mx, mn, de, b, nbin, mp = lim[g]
        assert (mx, mn, de, mp) == (d.gene_max[g], d.gene_min[g], d.gene_del[g], d.gene_map[g])
        assert b == 1.0 / nbin
    # set_bins by hand: a dihedral gene of -180..180 by 10 has 36 bins; the grid gene of 1..N-1
    # by 1, mapped, has N - 2 + 1
    assert results.set_bins(-180.0, 180.0, 10.0, 0) == (1.0 / 36.0, 36.0)
    assert results.set_bins(1.0, 1000.0, 1.0, 1) == (1.0 / 1000.0, 1000.0)
    # a fractional count gets one more bin added, not rounded: 360 / 7 + 1
    assert results.set_bins(-180.0, 180.0, 7.0, 0)[1] == 360.0 / 7.0 + 1.0
    assert data[5:5 + 48] == struct.pack("<5di4x", *lim[0])


# ---------------------------------------------------------------------------------------------
# GPU: fxe_cluster through the C ABI
# ---------------------------------------------------------------------------------------------

def assert_same(g, r, R):
    nc = r["n_clusters"]
    assert g["n_clusters"] == nc
    for k in ("top", "freq", "member_of"):
        np.testing.assert_array_equal(g[k], r[k], err_msg=k)
    np.testing.assert_array_equal(g["rmsd"].view(np.int32), r["rmsd"].view(np.int32))
    for k in ("tcf", "acf"):
        scale = np.maximum(1.0, np.abs(r[k]))
        assert (np.abs(g[k] - r[k]) / scale).max() <= 1e-12, k
    np.testing.assert_array_equal(g["top_rmsd"][:nc, :nc], r["top_rmsd"][:nc, :nc])


@pytest.mark.gpu
def test_gpu_cluster_golden(fixture):
    from flexaidds_gb300 import evaluator
    d, ic, e, cases, cads = fixture
    ev = evaluator.GPUEvaluator(d, max_poses=64)
    for (T, thr, R), cad in zip(cases, cads):
        g = ev.cluster(ic, e, T, thr, R)
        assert results.cad_text(g) == cad, (T, thr, R)
        assert_same(g, oracle_cluster(d, ic, e, T, thr, R), R)
    ev.close()


@pytest.mark.gpu
@pytest.mark.parametrize("T,thr,R", [(0, 2.0, 10), (300, 2.0, 10), (0, 1.5, 300), (298, 2.5, 64)])
def test_gpu_cluster_large(small_system, T, thr, R):
    from flexaidds_gb300 import evaluator
    _, d = small_system
    ic, e = synth.clustered_ensemble(d, 150, 120, seed=91, spread=3)
    ev = evaluator.GPUEvaluator(d, max_poses=64)
    g = ev.cluster(ic, e, T, thr, R)
    r = oracle_cluster(d, ic, e, T, thr, R)
    assert r["n_clusters"] == min(R, r["n_clusters"]) and r["freq"].sum() > R
    assert_same(g, r, R)
    assert ev.cluster_time() > 0.0
    ev.close()


@pytest.mark.gpu
def test_gpu_cluster_with_side_chains():
    """Rotamer genes select side chains only; the ligand's coordinates, and so the clusters, do not
    depend on them."""
    from flexaidds_gb300 import evaluator, prepare, system
    d = prepare.prepare(system.make_inputs(2000, 8.0, 24, 6, seed=43, side_chains=3))
    ic, e = synth.clustered_ensemble(d, 40, 50, seed=92)
    ev = evaluator.GPUEvaluator(d, max_poses=64)
    g = ev.cluster(ic, e, 300, 2.0, 20)
    assert_same(g, oracle_cluster(d, ic, e, 300, 2.0, 20), 20)
    ic2 = ic.copy()
    rot = np.nonzero(d.gene_typ == 4)[0]
    ic2[:, rot] = d.gene_max[rot]
    g2 = ev.cluster(ic2, e, 300, 2.0, 20)
    for k in ("top", "freq", "member_of", "rmsd", "acf"):
        np.testing.assert_array_equal(g2[k], g[k])
    ev.close()


@pytest.mark.gpu
def test_gpu_cluster_edges(small_system):
    from flexaidds_gb300 import evaluator
    _, d = small_system
    ic, e = synth.clustered_ensemble(d, 5, 20, seed=93)
    ev = evaluator.GPUEvaluator(d, max_poses=64)
    one = ev.cluster(ic[:1], e[:1], 0, 2.0, 10)
    assert one["n_clusters"] == 1 and one["top"][0] == 0 and one["freq"][0] == 1
    assert one["member_of"][0] == 0 and one["acf"][0] == e[0]
    for T, thr, R in [(0, 0.0, 1), (0, 1e9, 5), (300, 1e9, 4), (0, 0.0, 1000)]:
        assert_same(ev.cluster(ic, e, T, thr, R), oracle_cluster(d, ic, e, T, thr, R), R)
    # an IC outside its gene limits, a zero partition function, bad arguments
    bad = ic.copy()
    bad[3, 1] = d.gene_max[1] + 1.0
    with pytest.raises(evaluator.FxeError):
        ev.cluster(bad, e, 0, 2.0, 10)
    with pytest.raises(evaluator.FxeError):
        ev.cluster(ic, np.full_like(e, 1.0e6), 1, 2.0, 10)
    with pytest.raises(evaluator.FxeError):
        ev.cluster(ic, e, 0, -1.0, 10)
    with pytest.raises(evaluator.FxeError):
        ev.cluster(ic, e, 0, 2.0, 0)
    # the context still answers after the rejected calls
    assert_same(ev.cluster(ic, e, 0, 2.0, 10), oracle_cluster(d, ic, e, 0, 2.0, 10), 10)
    ev.close()


@pytest.mark.gpu
def test_gpu_cluster_of_a_ga_ensemble(small_system):
    """A GA job's ensemble (fxe_ga_ensemble: every generation's population, sorted, near-duplicates
    removed) clustered on the device, as the reference clusters chrom_snapshot after its GA."""
    from flexaidds_gb300 import evaluator
    from oracle import ga as ref_ga
    _, d = small_system
    P, G = 128, 4
    ev = evaluator.GPUEvaluator(d, max_poses=P)
    eng = evaluator.GAEngine(max_jobs=1)
    slot = eng.admit(eng.job(ev, P, G, 4242, 0.9, 0.02), ev)
    snaps = []
    for _ in range(G):
        eng.step()
        snaps.append(eng.read_population(slot, P))
    assert eng.finished() == [slot]
    ic, e = eng.ensemble(slot)
    # the restated assembly: snapshots sorted by energy (ties in snapshot order), a chromosome
    # dropped when every decoded gene is within 0.1 of the last one kept
    g_all = np.concatenate([s[0] for s in snaps])
    e_all = np.concatenate([s[1] for s in snaps])
    ic_all = ref_ga.clamped_ic(d, g_all)
    keep, last = [], None
    for i in np.argsort(e_all, kind="stable"):
        if last is None or not np.all(np.abs(ic_all[i] - last) < 0.1):
            keep.append(i)
            last = ic_all[i]
    np.testing.assert_array_equal(e, e_all[keep])
    np.testing.assert_array_equal(ic, ic_all[keep])
    _, best, th = eng.collect(slot, 300.0)
    assert th["n_ensemble"] == len(e) and best == e[0]
    for T in (0, 300):
        assert_same(ev.cluster(ic, e, T, 2.0, 10), oracle_cluster(d, ic, e, T, 2.0, 10), 10)
    ev.close()


# ---------------------------------------------------------------------------------------------
# Pose PDB files: the records of the reference's first result file (write_pdb after ic2cf of
# the head of cluster 0), rebuilt with the naming the pinning harness gives its atoms
# ---------------------------------------------------------------------------------------------

def harness_records(d, lig_bonds):
    """The atoms as the harness names them: receptor atom k (1-based) numbered k in residue "REC"
    of chain A, one residue per atom except the flexible side chains ("FLX", one residue each);
    ligand atoms 90001.. in residue "LIG" 1; names empty. Returns (receptor records of the
    rigid residues with their receptor indices, ligand records, ligand bond lists)."""
    first = {int(f): int(n) for f, n in zip(getattr(d, "flex_first", []), getattr(d, "flex_natm", []))}
    rec, nres, k = [], 0, 0
    while k < d.rec_type.shape[0]:
        nres += 1
        if k in first:
            k += first[k]
            continue
        rec.append((k, results.PdbAtom(k + 1, "", "REC", "A", nres, False, d.rec_type[k])))
        k += 1
    lig = [results.PdbAtom(90001 + i, "", "LIG", " ", 1, True, d.lig_type[i]) for i in range(d.n_lig)]
    adj = [[] for _ in range(d.n_lig)]
    for a, b in lig_bonds:
        adj[a].append(b)
        adj[b].append(a)
    return rec, lig, adj


def records_of(text):
    keep = []
    for line in text.splitlines():
        if line.startswith("HETATM") or line.startswith("CONECT") or line == "END":
            keep.append(line)
        elif line.startswith("ATOM  ") and line[17:20] == "REC":
            keep.append(line)
    return keep


def pose_text(d, z, lig_xyz):
    rec, lig, adj = harness_records(d, z["lig_bonds"])
    atoms = [a for _, a in rec] + lig
    xyz = np.concatenate([np.asarray(d.rec_xyz, np.float32).reshape(-1, 3)[[k for k, _ in rec]],
                          np.asarray(lig_xyz, np.float32).reshape(-1, 3)])
    nr = len(rec)
    return results.pose_pdb_text("REMARK optimized structure", atoms, xyz,
                                 ligand_bonds=[[nr + b for b in adj[i]] for i in range(d.n_lig)],
                                 ligand_atoms=list(range(nr, nr + d.n_lig)))


@pytest.mark.parametrize("name", CLUSTER_FIXTURES)
def test_pose_pdb_against_reference(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d, ic, e, cases, _ = load(name)
    T, thr, R = cases[0]
    top0 = int(oracle_cluster(d, ic, e, T, thr, R)["top"][0])
    xyz = port.Oracle(d).build_ic(ic[top0:top0 + 1])[0]
    ref = records_of(bytes(z["pdb_0"]).decode())
    mine = records_of(pose_text(d, z, xyz))
    assert len(ref) > d.n_lig * 2
    assert mine == ref


def test_element_table():
    """get_element's ranges (LIB/write_pdb.cpp:218-300)."""
    assert [results.element_of(t) for t in (1, 5, 6, 12, 13, 16, 17, 21)] == \
        [" C", " C", " N", " N", " O", " O", " S", " S"]
    assert results.element_of(24) == "Cl" and results.element_of(39) == "Du"
    assert results.element_of(40) == "  " and results.element_of(0) == "  "


@pytest.mark.gpu
@pytest.mark.parametrize("name", CLUSTER_FIXTURES)
def test_gpu_pose_pdb_against_reference(name):
    """The head of the first cluster, built by the device (fxe_eval_ic), written as a pose file:
    its records equal the reference's."""
    from flexaidds_gb300 import evaluator
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d, ic, e, cases, _ = load(name)
    T, thr, R = cases[0]
    ev = evaluator.GPUEvaluator(d, max_poses=64)
    top0 = int(ev.cluster(ic, e, T, thr, R)["top"][0])
    ev.eval_ic(ic[top0:top0 + 1])
    mine = records_of(pose_text(d, z, ev.ligand_xyz(0)))
    assert mine == records_of(bytes(z["pdb_0"]).decode())
    ev.close()


def test_clustered_ensemble_generator(tiny_system):
    """The seeded stand-in ensemble: sorted by energy, every IC on a bin and within its limits,
    rotamer genes untouched, the same for the same seed."""
    _, d = tiny_system
    ic, e = synth.clustered_ensemble(d, 7, 11, seed=3)
    assert ic.shape == (77, d.n_genes) and e.shape == (77,)
    assert np.all(np.diff(e) >= 0)
    assert np.all(ic >= d.gene_min) and np.all(ic <= d.gene_max)
    k = (ic - d.gene_min) / d.gene_del
    np.testing.assert_array_equal(ic, d.gene_min + d.gene_del * np.rint(k))
    ic2, e2 = synth.clustered_ensemble(d, 7, 11, seed=3)
    np.testing.assert_array_equal(ic, ic2)
    np.testing.assert_array_equal(e, e2)


def test_result_file_edges(tiny_system):
    _, d = tiny_system
    assert results.cad_text({"n_clusters": 0, "top": [], "freq": [], "tcf": [], "acf": [], "top_rmsd": []}) == ""
    with pytest.raises(ValueError):
        results.read_par(b"chrom" + bytes(10), d.n_genes)
    data = results.par_bytes(d, np.zeros((0, d.n_genes), np.int32))
    lim, genes = results.read_par(data, d.n_genes)
    assert len(lim) == d.n_genes and genes.shape == (0, d.n_genes)
    with pytest.raises(ValueError):
        results.par_bytes(d, np.zeros((3, d.n_genes + 1), np.int32))
    text = results.pose_pdb_text("REMARK x", [results.PdbAtom(1, " CA ", "ALA", "A", 7, False, 2)],
                                 [[1.0, -2.0, 3.5]])
    assert text == ("REMARK coordinate file generated by FlexAID\nREMARK x\n"
                    "ATOM      1  CA  ALA A   7       1.000  -2.000   3.500  1.00  0.00           C  \nEND\n")
