"""C ABI behaviour on the device: batching, device-resident entry points, errors, statmech."""
import ctypes as C
import math

import numpy as np
import pytest

from flexaidds_gb300 import capi, evaluator, synth
from oracle import port

pytestmark = pytest.mark.gpu

KB = 0.001987206


def test_chunked_batch_equals_single_launch(tiny_system):
    _, d = tiny_system
    genes = synth.random_genes(700, d.n_genes, seed=3)
    a = evaluator.GPUEvaluator(d, max_poses=1024).eval_genes(genes)
    b = evaluator.GPUEvaluator(d, max_poses=96).eval_genes(genes)   # 8 chunks
    np.testing.assert_array_equal(a, b)


def test_eval_ic_equals_eval_genes(tiny_system):
    _, d = tiny_system
    genes = synth.random_genes(300, d.n_genes, seed=4)
    ev = evaluator.GPUEvaluator(d, max_poses=512)
    np.testing.assert_array_equal(ev.eval_genes(genes), ev.eval_ic(d.genes_to_ic(genes)))


def test_device_entry_point_matches_host(tiny_system):
    torch = pytest.importorskip("torch")
    _, d = tiny_system
    genes = synth.random_genes(500, d.n_genes, seed=5)
    ev = evaluator.GPUEvaluator(d, max_poses=512)
    want = ev.eval_genes(genes)
    dg = torch.from_numpy(genes).cuda()
    dout = torch.zeros(500 * capi.CF_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    ev.eval_genes_device(dg.data_ptr(), 500, dout.data_ptr(), s.cuda_stream)
    s.synchronize()
    got = np.frombuffer(dout.cpu().numpy().tobytes(), capi.CF_DTYPE)
    np.testing.assert_array_equal(got, want)


def test_empty_batch_and_bad_arguments(tiny_system):
    _, d = tiny_system
    ev = evaluator.GPUEvaluator(d, max_poses=64)
    assert ev.eval_genes(np.zeros((0, d.n_genes), np.int32)).shape == (0,)
    lib = evaluator.load_library()
    assert lib.fxe_eval_genes(ev.handle, 4, None, None) == 1
    assert lib.fxe_eval_genes_device(ev.handle, 65, C.c_void_p(16), C.c_void_p(16), None) == 1
    assert lib.fxe_context_set_precision(ev.handle, 7) == 1
    with pytest.raises(evaluator.FxeError):
        ev.contacts(10_000, 0)
    assert "invalid" in lib.fxe_last_error().decode()


def test_polyhedron_failures_and_clashes_are_sentinels(small_system):
    _, d = small_system
    genes = synth.random_genes(4000, d.n_genes, seed=8)
    out = evaluator.GPUEvaluator(d, max_poses=4096).eval_genes(genes)
    clashed = out["status"] == 2
    failed = out["status"] == 1
    assert clashed.sum() > 100
    assert np.all(out["evalue"][clashed] >= 1e4)
    assert np.all(out["evalue"][failed] == 1e6 + 1.0)
    assert np.all(out["metal_coord"][clashed | failed] == 1.0)


# --- statmech ------------------------------------------------------------------------------

def _rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


@pytest.mark.parametrize("n", [1, 2, 1000, 1_000_000])
def test_thermo_against_fp64_oracle(n):
    rng = np.random.default_rng(n)
    e = rng.normal(-30.0, 4.0, n)
    m = rng.integers(1, 4, n).astype(np.int32)
    for mult in (None, m):
        got = evaluator.thermo(e, mult, 300.0)
        want = port.thermo(e, mult, 300.0)
        for k in ("log_Z", "free_energy", "mean_energy", "entropy", "heat_capacity"):
            assert _rel(got[k], want[k]) <= 1e-9, (k, got[k], want[k])
        # the reported forms: dG = F, dH = <E>, -T dS, Cv
        assert _rel(-300.0 * got["entropy"], -300.0 * want["entropy"]) <= 1e-9


def test_thermo_known_answers():
    th = evaluator.thermo([-10.0, -8.0], None, 300.0)
    beta = 1.0 / (KB * 300.0)
    z = math.exp(10 * beta) + math.exp(8 * beta)
    assert _rel(th["log_Z"], math.log(z)) <= 1e-12
    assert _rel(th["free_energy"], -KB * 300.0 * math.log(z)) <= 1e-12
    th = evaluator.thermo([-10.0] * 8, None, 300.0)
    assert _rel(th["entropy"], KB * math.log(8)) <= 1e-12
    th = evaluator.thermo([-500.0, 0.0], None, 300.0)
    assert all(math.isfinite(v) for v in th.values())


def test_boltzmann_weights_over_the_double_range():
    """Weights from 1 down past the double range against the host's exp: within 1e-12 where the
    weight is a normal double, 0 where it underflows."""
    e = np.linspace(-1000.0, 0.0, 20001)
    w = evaluator.boltzmann_weights(e, None, 300.0)
    beta = 1.0 / (KB * 300.0)
    lw = -beta * e
    m = lw.max()
    lnz = m + math.log(np.exp(lw - m).sum())
    want = np.exp(lw - lnz)
    normal = want > 1e-290
    assert normal.sum() > 5000 and (want == 0.0).sum() > 5000
    np.testing.assert_allclose(w[normal], want[normal], rtol=1e-12, atol=0.0)
    assert np.all(w[want == 0.0] == 0.0)
    assert np.all((w >= 0.0) & (w <= 1.0))


def test_boltzmann_weights_and_engine():
    rng = np.random.default_rng(9)
    e = rng.normal(-20.0, 2.0, 50_000)
    w = evaluator.boltzmann_weights(e, None, 310.0)
    np.testing.assert_allclose(w, port.thermo_weights(e, None, 310.0), rtol=1e-9, atol=1e-300)
    assert abs(w.sum() - 1.0) < 1e-12
    a, b = evaluator.StatMechEngine(300.0), evaluator.StatMechEngine(300.0)
    for x in (-15.0, -12.0):
        a.add_sample(x)
    for x in (-10.0, -8.0):
        b.add_sample(x)
    assert abs(a.delta_G(b) + b.delta_G(a)) < 1e-12
    assert abs(a.delta_G(b) - (a.compute()["free_energy"] - b.compute()["free_energy"])) < 1e-12


def test_thermo_device_form():
    torch = pytest.importorskip("torch")
    e = np.random.default_rng(2).normal(-25.0, 3.0, 200_000)
    de = torch.from_numpy(e).cuda()
    lib = evaluator.load_library()
    t = capi.Thermo()
    assert lib.fxe_thermo_compute_device(C.c_void_p(de.data_ptr()), None, e.size, 300.0, C.byref(t), None) == 0
    assert _rel(t.log_Z, port.thermo(e, None, 300.0)["log_Z"]) <= 1e-9


def test_thermo_rejects_bad_input():
    with pytest.raises(evaluator.FxeError):
        evaluator.thermo(np.zeros(0), None, 300.0)
    with pytest.raises(evaluator.FxeError):
        evaluator.thermo([-1.0], None, -5.0)
    with pytest.raises(evaluator.FxeError):
        evaluator.thermo([-1.0, -2.0], np.array([1, 0], np.int32), 300.0)
