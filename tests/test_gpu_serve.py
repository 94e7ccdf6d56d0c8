"""Serving with continuous batching: every job's result is the same alone and in the mix, and
admission under a memory budget that holds only a few jobs at a time still serves them all."""
import numpy as np
import pytest

from flexaidds_gb300 import prepare, serve, synth, system

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def requests():
    recs = {"A": system.make_inputs(1200, 7.0, 12, 3, seed=61), "B": system.make_inputs(900, 6.0, 12, 3, seed=62)}
    out = []
    rng = np.random.default_rng(3)
    for k in range(8):
        key = "A" if k % 3 else "B"
        base = recs[key]
        lig = synth.random_ligand(int(rng.integers(10, 30)), int(rng.integers(0, 6)), seed=500 + k)
        inp = system.SystemInputs(receptor=base.receptor, ligand=lig, grid_xyz=base.grid_xyz, emat=base.emat)
        out.append(serve.JobRequest(arrival=0.02 * k, receptor=key, inputs=inp, population=int(rng.integers(40, 160)),
                                    generations=int(rng.integers(2, 7)), seed=1000 + k))
    return out


def _same(a, b):
    assert a.best_energy == b.best_energy
    np.testing.assert_array_equal(a.best_genes, b.best_genes)
    for k in a.thermo:
        x, y = a.thermo[k], b.thermo[k]
        assert x == y or abs(x - y) <= 1e-12 * abs(y), k


def test_each_job_same_alone_and_in_the_mix(requests):
    srv = serve.DockingServer(max_jobs=8)
    mixed = {r.index: r for r in srv.run(requests)}
    srv.close()
    assert sorted(mixed) == list(range(len(requests)))
    for i, req in enumerate(requests):
        solo = serve.DockingServer(max_jobs=1)
        alone = solo.run([serve.JobRequest(0.0, req.receptor, req.inputs, req.population, req.generations, req.seed)])
        solo.close()
        _same(mixed[i], alone[0])
    s = serve.latency_summary(list(mixed.values()))
    assert s["p50_s"] <= s["p95_s"] <= s["p99_s"]


def test_admission_under_a_small_budget(requests):
    one = serve.context_bytes(prepare.prepare(requests[0].inputs), 160) * 2.5
    srv = serve.DockingServer(max_jobs=8, hbm_budget=one)
    res = srv.run(requests)
    srv.close()
    assert len(res) == len(requests)
    # with room for about two jobs, later arrivals wait for admission
    assert max(r.admitted - r.arrival for r in res) > 0.0


def test_receptor_cache_prepares_on_the_device(requests):
    """The server's receptor set-up (cleft grid and ICs generated on the device) matches the host
    restatement: the same grid points, ICs within two units in the last place."""
    srv = serve.DockingServer(max_jobs=2)
    r = requests[0]
    setup, xyz, _ = srv._receptor(r.receptor, r.inputs)
    np.testing.assert_array_equal(xyz, r.inputs.grid_xyz)
    host = prepare.cleft_ic(r.inputs.grid_xyz, setup[0][0])
    ulps = np.abs(setup[1].view(np.int32).astype(np.int64) - host.view(np.int32).astype(np.int64))
    assert ulps.max() <= 2
    srv.close()
