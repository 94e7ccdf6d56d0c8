"""Reference precision against the oracle over a spread of seeded systems: receptor sizes and
clefts, ligand sizes and torsions, flexible side chains, intramolecular terms on and off, and
density-curve energy entries. Statuses must agree on every pose and scores within 1e-9 on every
scored pose."""
import importlib.util
import os

import numpy as np
import pytest

from flexaidds_gb300 import evaluator, prepare, synth, system
from oracle import port

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# (receptor atoms, cleft radius, ligand atoms, torsions, seed, side chains, intramolecular, curves)
CASES = [
    (2000, 8.0, 24, 6, 101, 0, 1, False), (2000, 8.0, 24, 6, 102, 3, 1, False),
    (900, 7.0, 16, 4, 103, 2, 0, True), (4000, 10.0, 36, 8, 104, 4, 1, False),
    (600, 6.0, 10, 2, 106, 2, 0, False), (3000, 9.0, 30, 10, 107, 3, 1, True),
]


def _density_curves():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.density_curves


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}rec-{c[2]}lig-{c[5]}sc")
def test_reference_precision_sweep(case):
    n_rec, cleft, n_lig, n_tor, seed, sc, intra, curves = case
    inp = system.make_inputs(n_rec, cleft, n_lig, n_tor, seed=seed, side_chains=sc)
    inp.intramolecular = intra
    if curves:
        _density_curves()(inp, seed)
    d = prepare.prepare(inp)
    genes = synth.random_genes(3000, d.n_genes, seed=seed + 1)
    port.set_reference_compat(True)
    port.set_trig_rounding(False)
    r = port.Oracle(d).eval_ic(d.genes_to_ic(genes))["cf"]
    ev = evaluator.GPUEvaluator(d, max_poses=3000)
    g = ev.eval_genes(genes)
    np.testing.assert_array_equal(g["status"], r["status"])
    ok = g["status"] == 0
    assert ok.sum() >= 10
    rel = np.abs(g["evalue"] - r["evalue"]) / np.maximum(1.0, np.abs(r["evalue"]))
    assert rel[ok].max() <= 1e-9
    assert rel[~ok].max() <= 1e-6 if (~ok).any() else True
    assert ev.stats()["capacity"] == 0
    ev.close()
