"""The polyhedron launch's autotuner (fxe_context_autotune): it picks an occupancy cap within the
SM's capacity for the context's size class, the process-wide table returns it for that class only,
and the records do not change with it."""
import numpy as np
import pytest

from flexaidds_gb300 import evaluator, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1])
def test_autotune_picks_a_cap_and_keeps_results(small_system, prec):
    import torch
    _, d = small_system
    genes = synth.random_genes(1024, d.n_genes, seed=21)
    ev = evaluator.GPUEvaluator(d, max_poses=1024, precision=prec)
    before = ev.eval_genes(genes)
    dg = torch.from_numpy(np.ascontiguousarray(genes)).cuda()
    cap, ms = ev.autotune(dg.data_ptr(), genes.shape[0], reps=2)
    torch.cuda.synchronize()
    assert cap >= 1 and ms > 0.0
    mobile = d.n_sc + d.n_lig
    assert evaluator.autotune_lookup(prec, mobile, genes.shape[0]) == cap
    assert evaluator.autotune_lookup(prec, mobile, 100_000) == 0          # another class: untouched
    after = ev.eval_genes(genes)
    assert after.tobytes() == before.tobytes()
    ev.close()


def test_autotune_sweep_reports_every_cap(small_system):
    """fxe_context_autotune_sweep: one entry per cap from half the SM's capacity to all of it, the
    fastest recorded in the table."""
    import torch
    _, d = small_system
    genes = synth.random_genes(512, d.n_genes, seed=22)
    ev = evaluator.GPUEvaluator(d, max_poses=512, precision=0)
    dg = torch.from_numpy(np.ascontiguousarray(genes)).cuda()
    sweep = ev.autotune_sweep(dg.data_ptr(), genes.shape[0], reps=1)
    caps = sorted(sweep)
    assert caps and caps == list(range(caps[0], caps[-1] + 1)) and caps[0] >= 1
    assert all(ms > 0.0 for ms in sweep.values())
    best = min(caps, key=lambda c: (sweep[c], c))
    assert evaluator.autotune_lookup(0, d.n_sc + d.n_lig, genes.shape[0]) == best
    ev.close()


@pytest.mark.parametrize("which", ["tiny", "small", "scale"])
def test_cell_staging_keeps_records(tiny_system, small_system, which):
    """The contact scan with the rigid cell entries staged in shared memory by bulk copies gives
    the records of the scan that reads them in place, bit for bit, on single contexts."""
    if which == "scale":
        # the benchmark's 6,000-atom system with three side chains, where most uniform poses
        # clash: its first population of poses that pass the clash pre-filter
        import bench
        d = bench.make_system()
        filt = evaluator.GPUEvaluator(d, max_poses=100_000, precision=1)
        genes = bench.scored_populations(d, 1, lambda g: filt.eval_genes(g)["status"])[0][:1024]
        filt.close()
    else:
        d = (tiny_system if which == "tiny" else small_system)[1]
        genes = synth.random_genes(1024, d.n_genes, seed=23)
    recs = []
    for mode in (evaluator.GPUEvaluator.CELLS_IN_PLACE, evaluator.GPUEvaluator.CELLS_STAGED):
        ev = evaluator.GPUEvaluator(d, max_poses=1024, precision=0, cell_staging=mode)
        recs.append(ev.eval_genes(genes))
        ev.close()
    assert (recs[0]["status"] == 0).sum() > 10
    assert recs[0].tobytes() == recs[1].tobytes()


def test_cell_staging_in_batches(small_system):
    """Batched launches take the contexts' common setting: staged and in-place batches agree."""
    _, d = small_system
    genes = [synth.random_genes(300 + 100 * k, d.n_genes, seed=30 + k) for k in range(3)]
    outs = []
    for mode in (evaluator.GPUEvaluator.CELLS_IN_PLACE, evaluator.GPUEvaluator.CELLS_STAGED):
        evs = [evaluator.GPUEvaluator(d, max_poses=512, precision=0, cell_staging=mode) for _ in genes]
        b = evaluator.Batch(max_jobs=4, max_poses=2048)
        outs.append(b.eval_genes(list(zip(evs, genes))))
        b.close()
        for ev in evs:
            ev.close()
    for a, b in zip(*outs):
        assert a.tobytes() == b.tobytes()


def test_autotune_contacts_times_both_forms(small_system):
    """fxe_context_autotune_contacts: both forms timed, the faster recorded; the automatic setting
    then keeps the records."""
    import torch
    _, d = small_system
    genes = synth.random_genes(1024, d.n_genes, seed=24)
    ev = evaluator.GPUEvaluator(d, max_poses=1024, precision=0)
    before = ev.eval_genes(genes)
    dg = torch.from_numpy(np.ascontiguousarray(genes)).cuda()
    t = ev.autotune_contacts(dg.data_ptr(), genes.shape[0], reps=3)
    torch.cuda.synchronize()
    print("contacts launch over 1,024 poses:", t)
    assert t["in_place_ms"] > 0.0 and t["staged_ms"] > 0.0
    assert t["staged"] == (t["staged_ms"] < t["in_place_ms"])
    assert ev.eval_genes(genes).tobytes() == before.tobytes()
    ev.close()
