"""Host-side pieces that need no GPU: generators, set-up, gene decode, the C ABI's library."""
import ctypes as C
import importlib.util
import os
import re

import numpy as np
import pytest

from flexaidds_gb300 import capi, prepare, synth, system

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _make_golden():
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


# --- generators -----------------------------------------------------------------------------

def test_receptor_generator_is_seeded_and_poisson():
    a = synth.poisson_disc_receptor(600, 6.0, seed=3)
    b = synth.poisson_disc_receptor(600, 6.0, seed=3)
    np.testing.assert_array_equal(a.xyz, b.xyz)
    np.testing.assert_array_equal(a.type, b.type)
    assert a.xyz.shape == (600, 3) and a.type.min() >= 1 and a.type.max() <= 40
    d2 = ((a.xyz[:, None, :] - a.xyz[None, :, :]) ** 2).sum(-1)
    d2[np.arange(600), np.arange(600)] = 1e9
    assert np.sqrt(d2.min()) >= 2.8 - 1e-4
    assert np.linalg.norm(a.xyz - a.cleft_center, axis=1).min() >= 6.0


def test_ligand_generator_geometry():
    lig = synth.random_ligand(24, 6, seed=7)
    assert lig.xyz.shape == (24, 3)
    for i, j in lig.bonds:
        assert abs(np.linalg.norm(lig.xyz[i] - lig.xyz[j]) - 1.53) < 1e-3
    assert sum(1 for f in lig.flex if len(f)) == 6


# --- set-up restatement against the reference's own set-up (golden descriptors) ---------------

@pytest.mark.parametrize("name", ["c0_2000_24", "curves_900_16", "outside_600_10", "scale_6000_48",
                                  "flex_2000_24", "flexcurves_900_16"])
def test_prepare_matches_reference_setup(name):
    from conftest import load_golden
    dref, _ = load_golden(name)
    d = prepare.prepare(_make_golden().inputs_for(name))
    for k in ("lig_rec", "build_order", "bonded", "gene_typ", "gene_atm", "gene_map", "rec_type",
              "lig_type", "emat_weight", "emat_off", "flex_first", "flex_natm", "flex_nrot",
              "flex_isbb", "flex_xyz", "flex_bonded"):
        np.testing.assert_array_equal(getattr(d, k), getattr(dref, k), err_msg=k)
    for k in ("gene_min", "gene_max", "gene_del", "emat_x", "emat_y", "rec_xyz", "rec_radius",
              "lig_radius"):
        np.testing.assert_array_equal(getattr(d, k), getattr(dref, k), err_msg=k)
    # float geometry of buildic / calc_center / calc_cleftic: the restatement rounds the same
    # expressions in a different order in places
    for k, tol in (("ori", 1e-5), ("globalmin", 1e-5), ("globalmax", 1e-5), ("lig_ic", 1e-3),
                   ("lig_shift", 1e-3), ("grid_ic", 1e-3)):
        np.testing.assert_allclose(getattr(d, k), getattr(dref, k), atol=tol, err_msg=k)


# --- gene decode (genetoic, LIB/gaboom.cpp:2887-2906) ------------------------------------------

def _genetoic_walk(gmin, gmax, gdel, gmap, gene):
    """The reference's linear walk, written out: tot += bin until tot >= u."""
    nbin = (gmax - gmin) / gdel
    if nbin - int(nbin) > 0.0:
        nbin += 1.0
    if gmap:
        nbin += 1.0
    b = 1.0 / nbin
    u = gene / (2147483647.0 + 1.0)
    tot, i = b, 0
    while tot < u:
        tot += b
        i += 1
    return gmin + gdel * i


@pytest.mark.parametrize("lim", [(-180.0, 180.0, 10.0, 0), (0.0, 180.0, 5.0, 0), (1.0, 4095.0, 1.0, 1),
                                 (-180.0, 175.0, 5.0, 0)])
def test_gene_decode_matches_linear_walk(lim):
    tab = system.gene_bins(*lim)
    rng = np.random.default_rng(1)
    genes = np.concatenate([[0, 1, 2147483647, 1073741824], rng.integers(0, 2 ** 31, 3000)])
    u = genes.astype(np.float64) / 2147483648.0
    got = lim[0] + lim[2] * np.searchsorted(tab, u, side="left")
    want = np.array([_genetoic_walk(*lim, int(g)) for g in genes])
    np.testing.assert_array_equal(got, want)


# --- the C ABI's library ------------------------------------------------------------------------

def _declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "fxe.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    hdr = re.sub(r"//[^\n]*", "", hdr)
    return sorted(set(re.findall(r"\b(fxe_[a-z0-9_]+)\s*\(", hdr)))


@pytest.fixture(scope="module")
def libfxe():
    from flexaidds_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()
    return C.CDLL(build.LIB)


def test_library_exports_every_declared_symbol(libfxe):
    names = _declared_symbols()
    assert len(names) >= 12
    missing = [n for n in names if not hasattr(libfxe, n)]
    assert not missing, missing


def test_library_reports_errors_without_device(libfxe):
    """Entry points validate their arguments before touching a device."""
    libfxe.fxe_last_error.restype = C.c_char_p
    libfxe.fxe_context_create.argtypes = [C.c_void_p] * 4 + [C.c_int32, C.c_void_p]
    out = C.c_void_p()
    rc = libfxe.fxe_context_create(None, None, None, None, 16, C.byref(out))
    assert rc == 1 and out.value is None
    assert b"null" in libfxe.fxe_last_error().lower()


def test_struct_layouts_match_header():
    assert C.sizeof(capi.CF) == 11 * 8 + 2 * 4
    assert capi.CF_DTYPE.itemsize == C.sizeof(capi.CF)
    assert C.sizeof(capi.Thermo) == 8 * 8


# --- GA restatement ---------------------------------------------------------------------------

def test_ga_job_layout_matches_header():
    from flexaidds_gb300 import evaluator
    assert C.sizeof(evaluator.GAJob) == 136
    assert evaluator.GAJob.duplicates.offset == 88
    assert evaluator.GAJob.fitness.offset == 92
    assert evaluator.GAJob.temperature.offset == 128


def test_hash_genes_signature_known_answers():
    """hash_genes folds (int32_t)(to_ic + 0.5), sign-extended, into h with the boost-style mix."""
    from oracle import ga
    assert ga.signature([0.0]) == 0x9E3779B9
    assert ga.signature([-1.7]) == 0x9E3779B8            # (int32_t)(-1.2) = -1 wraps to 2^64 - 1
    h1 = 0x9E3779B9 + 3
    assert ga.signature([2.6, 0.2]) == h1 ^ ((0x9E3779B9 + (h1 << 6) + (h1 >> 2)) & ga.M64)


def test_ga_rejection_keeps_signatures_unique():
    from oracle import ga
    d = prepare.prepare(system.make_inputs(600, 6.0, 10, 2, seed=4))
    rej = ga.Rejector(d)
    pop = ga.initial_genes(77, 64, d.n_genes, rej)
    sigs = {ga.signature(r) for r in d.genes_to_ic(pop)}
    assert len(sigs) == 64
    for gen in range(3):
        child = ga.breed(pop, gen, 77, 0.9, 0.001, rej=rej)
        csig = [ga.signature(r) for r in d.genes_to_ic(child)]
        assert len(set(csig)) == len(csig) and not sigs.intersection(csig)
        sigs.update(csig)
        pop = child
    assert rej.rejected > 0 and len(rej.seen) == len(sigs)
    # allowing duplicates takes the candidates in order
    free = ga.breed(pop, 5, 77, 0.9, 0.001, rej=ga.Rejector(d, allow=True))
    np.testing.assert_array_equal(free, ga.breed(pop, 5, 77, 0.9, 0.001))


def test_fitness_models_restated():
    """sig_share from the gene limits; PSHARE divides the rank by a niche count of at least one
    and walks the population in fitness order after a generation; SMFREE with no temperature
    ranks only."""
    import math
    from oracle import ga
    d = prepare.prepare(system.make_inputs(600, 6.0, 10, 2, seed=4))
    ng = d.n_genes
    want = math.sqrt(sum((d.gene_max[g] - d.gene_min[g]) ** 2 for g in range(ng)) / ng)
    want /= 2.0 * 5.0 ** (1.0 / ng)
    assert abs(ga.sig_share(d) - want / 10.0) <= 1e-12 * want
    pop = ga.initial_genes(9, 24, ng)
    pe = np.sort(np.random.default_rng(1).normal(size=24))
    lin = ga.Fitness(pop, pe, d, "LINEAR")
    assert lin.fit == [float(24 - i) for i in range(24)] and lin.total == 300.0
    first = ga.Fitness(pop, pe, d, "PSHARE", initial=True)
    later = ga.Fitness(pop, pe, d, "PSHARE")
    assert first.order == list(range(24))
    assert all(f <= 24 - i for i, f in enumerate(first.fit))
    assert sorted(first.fit, reverse=True) == later.fit
    assert later.cum[-1] == later.total
    flat = ga.Fitness(pop, pe, d, "SMFREE", temperature=0.0)
    assert flat.fit == lin.fit


def test_side_chain_descriptors_are_validated(libfxe):
    """The ABI rejects inconsistent side-chain descriptors before it looks for a device."""
    import copy
    from flexaidds_gb300 import capi as ca
    libfxe.fxe_last_error.restype = C.c_char_p
    libfxe.fxe_context_create.argtypes = [C.c_void_p] * 4 + [C.c_int32, C.c_void_p]
    d = prepare.prepare(system.make_inputs(600, 6.0, 10, 2, seed=4, side_chains=2))

    def create(dd):
        pk = ca.Packed(dd)
        out = C.c_void_p()
        rc = libfxe.fxe_context_create(C.byref(pk.rec), C.byref(pk.lig), C.byref(pk.emat),
                                       C.byref(pk.params), 16, C.byref(out))
        return rc, libfxe.fxe_last_error().decode()

    bad = copy.deepcopy(d)
    bad.flex_xyz = bad.flex_xyz.copy()
    bad.flex_xyz[0, 0] += 0.5                       # rotamer 0 differs from the receptor
    rc, msg = create(bad)
    assert rc == 1 and "rotamer 0" in msg
    bad = copy.deepcopy(d)
    bad.gene_max = bad.gene_max.copy()
    bad.gene_max[-1] = float(bad.flex_nrot[-1])      # one past the last rotamer
    rc, msg = create(bad)
    assert rc == 1 and "rotamer gene limits" in msg
    bad = copy.deepcopy(d)
    bad.gene_atm = bad.gene_atm.copy()
    bad.gene_atm[-1] = 5                             # no such side chain
    rc, msg = create(bad)
    assert rc == 1 and "names no flexible side chain" in msg
    bad = copy.deepcopy(d)
    bad.flex_prob = np.asarray([1.5, 0.2], np.float32)
    rc, msg = create(bad)
    assert rc == 1 and "prob" in msg
    # the valid descriptor gets past validation (and stops at the missing device here)
    rc, msg = create(d)
    assert rc in (0, 7)


def test_energy_matrix_file_format(tmp_path):
    """read_emat takes the reference's upper-triangle lines: single values and density curves."""
    lines = []
    t = 3
    for i in range(t):
        for j in range(i, t):
            if (i, j) == (0, 2):
                lines.append(f"{i + 1:7d}-{j + 1:2d} =   0.0 -1.5  0.4 2.25  1.0 0.5")
            else:
                lines.append(f"{i + 1:7d}-{j + 1:2d} = {10.0 * i - j:8.1f}")
    p = tmp_path / "emat.dat"
    p.write_text("\n".join(lines) + "\n")
    emat, w, curves = system.read_emat(str(p))
    assert emat.shape == (3, 3) and w[0, 2] == 0 and w[2, 0] == 0 and w.sum() == 7
    assert emat[1, 2] == emat[2, 1] == np.float32(8.0)
    assert curves[(0, 2)] == [(0.0, -1.5), (0.4000000059604645, 2.25), (1.0, 0.5)]
    bad = tmp_path / "bad.dat"
    bad.write_text("\n".join(lines[:5]) + "\n")
    with pytest.raises(ValueError):
        system.read_emat(str(bad))


def _reference_file(*parts):
    from oracle import ref
    return os.path.join(ref.REFERENCE_ROOT, *parts)


@pytest.mark.skipif(not os.path.exists(_reference_file("WRK", "MC_st0r5.2_6.dat")),
                    reason="the reference checkout is not present")
def test_reference_energy_matrix_file_reads():
    emat, w, curves = system.read_emat(_reference_file("WRK", "MC_st0r5.2_6.dat"))
    assert emat.shape == (40, 40) and int(w.sum()) + 2 * len(curves) - sum(1 for (i, j) in curves if i == j) == 1600


def test_roulette_restatement_edges():
    """roulette_wheel: the first running sum above u * total, the last position when rounding
    leaves none above it, a uniform position when the total is not positive
    (LIB/gaboom.cpp:1158-1186)."""
    from oracle import ga
    f = ga.Fitness(np.zeros((4, 2), np.int32), np.zeros(4), None, "LINEAR")
    assert f.fit == [4.0, 3.0, 2.0, 1.0] and f.cum == [4.0, 7.0, 9.0, 10.0]
    assert [f.roulette(u) for u in (0.0, 0.39, 0.4, 0.69, 0.7, 0.89, 0.9, 0.999)] == [0, 0, 1, 1, 2, 2, 3, 3]
    f.cum, f.total = [0.0, 0.0, 0.0, 0.0], 0.0
    assert [f.roulette(u) for u in (0.0, 0.3, 0.6, 0.99)] == [0, 1, 2, 3]
