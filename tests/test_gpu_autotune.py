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
