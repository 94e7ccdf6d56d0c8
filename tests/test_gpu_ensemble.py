"""The GA ensemble assembled on the device (fxe_ensemble_dedup, and fxe_ga_collect /
fxe_ga_ensemble on a job's snapshots): energy sort and remove_dups against the reference's known
answers (tests/test_gaboom.cpp:309-372) and against the restatement in oracle/ga.py on random
ensembles built to hold long runs of identical chromosomes, near-duplicates and tied energies."""
import numpy as np
import pytest

from flexaidds_gb300 import evaluator
from oracle import ga

pytestmark = pytest.mark.gpu


def want(ic, e):
    order = np.argsort(e, kind="stable")
    kept = ga.remove_dups(ic[order])
    return order[kept]


@pytest.mark.parametrize("rows,kept", [
    ([[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]], 3),          # AllUnique
    ([[1.0, 2.0]] * 4, 1),                              # AllIdentical
    ([[1.0], [1.0], [5.0], [5.0]], 2),                  # SomeDuplicates
    ([[1.0, 2.0]], 1),                                  # SingleChromosome
    ([[1.0], [1.1]], 2),                                # ToleranceBoundary
    ([[1.0], [1.05]], 1),                               # WithinTolerance
])
def test_remove_dups_known_answers(rows, kept):
    ic = np.array(rows, np.float64)
    r = evaluator.ensemble_dedup(ic, np.zeros(len(rows)))
    assert len(r["index"]) == kept
    np.testing.assert_array_equal(r["index"], want(ic, np.zeros(len(rows))))


def synthetic(rng, n_unique, n, ng, run_max, near_frac):
    """Chromosomes on a 0.05 grid (so near-duplicates within 0.1 occur), repeated in runs of up
    to run_max copies (survivors across generations), energies tied within each copy."""
    base = np.round(rng.normal(size=(n_unique, ng)) * 2.0 / 0.05) * 0.05
    near = rng.random(n_unique) < near_frac
    base[near] = base[np.maximum(np.nonzero(near)[0] - 1, 0)] + 0.05 * rng.integers(-1, 2, size=(near.sum(), ng))
    e_base = np.round(rng.normal(size=n_unique) * 5.0, 2)
    reps = rng.integers(1, run_max + 1, size=n_unique)
    pick = np.repeat(np.arange(n_unique), reps)[:n]
    rng.shuffle(pick)
    return base[pick], e_base[pick]


@pytest.mark.parametrize("n_unique,n,ng,run_max,near", [
    (50, 400, 3, 40, 0.5),          # runs longer than the bounded scan
    (3000, 20000, 19, 8, 0.3),
    (20000, 200000, 12, 20, 0.1),
    (10, 1000, 2, 200, 0.9),        # almost everything near one chromosome
])
def test_random_ensembles_against_restatement(n_unique, n, ng, run_max, near):
    rng = np.random.default_rng(n_unique + n)
    ic, e = synthetic(rng, n_unique, n, ng, run_max, near)
    r = evaluator.ensemble_dedup(ic, e)
    w = want(ic, e)
    np.testing.assert_array_equal(r["index"], w)
    np.testing.assert_array_equal(r["energy"], e[w])


def test_special_energies():
    ic = np.arange(12, dtype=np.float64).reshape(6, 2)
    e = np.array([np.inf, -0.0, 0.0, -1e300, np.nan, 3.0])
    r = evaluator.ensemble_dedup(ic, e)
    # -1e300, -0 and +0 tied in input order, 3, inf, then NaN
    np.testing.assert_array_equal(r["index"], [3, 1, 2, 5, 0, 4])


def test_sizes_one_and_two():
    r = evaluator.ensemble_dedup(np.zeros((1, 4)), np.array([2.0]))
    np.testing.assert_array_equal(r["index"], [0])
    r = evaluator.ensemble_dedup(np.array([[0.0], [0.2]]), np.array([1.0, -1.0]))
    np.testing.assert_array_equal(r["index"], [1, 0])
