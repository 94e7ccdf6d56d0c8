"""Batched launches and the receptor cache: several contexts' populations in one launch of each
kernel give the records each context gives alone."""
import numpy as np
import pytest

from flexaidds_gb300 import evaluator, prepare, synth, system

pytestmark = pytest.mark.gpu


def _ligand_variant(inp, n_lig, n_tor, seed):
    """The same receptor and matrix with another seeded ligand."""
    lig = synth.random_ligand(n_lig, n_tor, seed=seed)
    return system.SystemInputs(receptor=inp.receptor, ligand=lig, grid_xyz=inp.grid_xyz, emat=inp.emat)


@pytest.fixture(scope="module")
def jobs_on_one_receptor():
    base = system.make_inputs(1500, 7.0, 12, 3, seed=71)
    shapes = [(12, 3), (20, 5), (9, 0), (31, 8), (16, 2)]
    descs = [prepare.prepare(_ligand_variant(base, n, t, 100 + k)) for k, (n, t) in enumerate(shapes)]
    sizes = [300, 41, 700, 5, 256]
    genes = [synth.random_genes(m, d.n_genes, seed=200 + k) for k, (d, m) in enumerate(zip(descs, sizes))]
    return descs, genes


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_equals_single_contexts(jobs_on_one_receptor, prec):
    descs, genes = jobs_on_one_receptor
    alone = [evaluator.GPUEvaluator(d, max_poses=1024, precision=prec).eval_genes(g) for d, g in zip(descs, genes)]
    first = evaluator.GPUEvaluator(descs[0], max_poses=1024, precision=prec)
    evs = [first] + [evaluator.GPUEvaluator(d, max_poses=1024, precision=prec, share_receptor_with=first)
                     for d in descs[1:]]
    batch = evaluator.Batch(max_jobs=8, max_poses=4096, max_genes=32)
    for _ in range(2):   # twice: the job table and staging are reused
        outs = batch.eval_genes(list(zip(evs, genes)))
        for a, b in zip(outs, alone):
            np.testing.assert_array_equal(a, b)
    assert batch.take_launches() == 8   # build, contacts, order, polyhedra; twice
    assert sum(int((o["status"] == 0).sum()) for o in outs) > 20


def test_batch_over_receptors_and_device_pointers():
    torch = pytest.importorskip("torch")
    from flexaidds_gb300 import capi
    specs = [(900, 6.0, 14, 4, 81), (1300, 7.0, 22, 6, 82), (700, 6.0, 10, 1, 83)]
    descs = [prepare.prepare(system.make_inputs(*sp[:4], seed=sp[4])) for sp in specs]
    genes = [synth.random_genes(400 + 50 * k, d.n_genes, seed=90 + k) for k, d in enumerate(descs)]
    evs = [evaluator.GPUEvaluator(d, max_poses=512) for d in descs]
    alone = [ev.eval_genes(g) for ev, g in zip(evs, genes)]
    dg = [torch.from_numpy(g).cuda() for g in genes]
    do = [torch.zeros(g.shape[0] * capi.CF_DTYPE.itemsize, dtype=torch.uint8, device="cuda") for g in genes]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    batch = evaluator.Batch(max_jobs=4, max_poses=2048, max_genes=32)
    batch.eval_genes_device([(ev, g.shape[0], d.data_ptr(), o.data_ptr()) for ev, g, d, o in zip(evs, genes, dg, do)],
                            s.cuda_stream)
    s.synchronize()
    for o, want in zip(do, alone):
        np.testing.assert_array_equal(np.frombuffer(o.cpu().numpy().tobytes(), capi.CF_DTYPE), want)


def test_batch_rejects_bad_jobs(jobs_on_one_receptor):
    descs, genes = jobs_on_one_receptor
    ev = evaluator.GPUEvaluator(descs[0], max_poses=64)
    batch = evaluator.Batch(max_jobs=2, max_poses=128, max_genes=32)
    with pytest.raises(evaluator.FxeError):          # n above the context's max_poses
        batch.eval_genes([(ev, genes[0][:100])])
    with pytest.raises(evaluator.FxeError):          # one context twice
        batch.eval_genes([(ev, genes[0][:10]), (ev, genes[0][10:20])])
    with pytest.raises(evaluator.FxeError):          # more jobs than max_jobs
        ev2 = evaluator.GPUEvaluator(descs[1], max_poses=64)
        ev3 = evaluator.GPUEvaluator(descs[2], max_poses=64)
        batch.eval_genes([(ev, genes[0][:4]), (ev2, genes[1][:4]), (ev3, genes[2][:4])])
