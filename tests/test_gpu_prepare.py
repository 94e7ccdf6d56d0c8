"""Receptor preparation on the device (fxe_cleft_grid; the steady cell list built at context
creation) against the host restatements of generate_grid and calc_cleftic and against the
reference's own set-up output held in the golden fixtures."""
import numpy as np
import pytest

from flexaidds_gb300 import evaluator, prepare, synth

pytestmark = pytest.mark.gpu


def snap(v):
    """GridKey's std::round(v * 1000) (halves away from zero)."""
    x = (np.asarray(v, np.float32) * np.float32(1000.0)).astype(np.float64)
    return (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64)


def host_grid(centers, radii, spacing=0.375):
    """generate_grid over several spheres: each sphere's lattice points (synth.cleft_grid, one
    sphere), minus points whose snapped key an earlier sphere produced."""
    seen, out = set(), []
    for c, r in zip(centers, radii):
        pts = synth.cleft_grid(np.asarray(c, np.float32), float(r), spacing)
        keys = [tuple(k) for k in snap(pts)]
        keep = [i for i, k in enumerate(keys) if k not in seen]
        out.append(pts[keep])
        seen.update(keys)
    return np.concatenate(out)


def test_single_sphere_grid_matches_host():
    c = np.array([1.2345, -7.5, 20.0625], np.float32)
    ori = np.array([0.5, 0.25, -1.0], np.float32)
    xyz, ic = evaluator.cleft_grid(c, [12.0], 0.375, ori)
    want = synth.cleft_grid(c, 12.0, 0.375)
    assert xyz.shape[0] == want.shape[0] > 130_000
    np.testing.assert_array_equal(xyz, want)
    # calc_cleftic: the host restatement rounds the same double-precision acos/atan2 once
    host = prepare.cleft_ic(want, ori)
    diff = (ic != host).any(axis=1)
    assert diff.sum() <= 10, diff.sum()
    ulps = np.abs(ic.view(np.int32).astype(np.int64) - host.view(np.int32).astype(np.int64))
    assert ulps.max() <= 1


def test_overlapping_spheres_drop_repeated_points():
    centers = np.array([[0.0, 0.0, 0.0], [3.1, 0.2, -1.0], [0.0, 0.0, 0.0], [-6.0, 4.0, 2.5]], np.float32)
    radii = np.array([5.0, 4.0, 2.0, 3.0], np.float32)
    xyz, _ = evaluator.cleft_grid(centers, radii, 0.375, [0.0, 0.0, 0.0])
    np.testing.assert_array_equal(xyz, host_grid(centers, radii))


def test_integer_spacing_branch():
    c = np.array([2.3, -1.1, 0.7], np.float32)
    xyz, _ = evaluator.cleft_grid(c, [3.0], 0.5, [0.0, 0.0, 0.0])
    # 1/0.5 is an integer: the lattice starts at (int)(c - r - s) (LIB/generate_grid.cpp:44-51)
    lo = [np.float32(int(np.float32(np.float32(c[k] - np.float32(3.0)) - np.float32(0.5)))) for k in range(3)]
    assert np.all(xyz.min(axis=0) >= np.asarray(lo, np.float32))
    d = xyz - c
    assert np.all((d * d).sum(axis=1) < 9.0 + 1e-4)
    assert xyz.shape[0] > 400


@pytest.mark.parametrize("name", ["c0_2000_24", "scale_6000_48"])
def test_grid_against_reference_setup(name):
    """The fixture's cleft sphere regenerated on the device: the reference's grid points (its own
    set-up made the fixture) exactly, and its calc_cleftic output within two units in the last
    place (the reference's acosf/atan2f round differently on about a fifth of the points, and the
    angle's conversion to degrees can double a one-unit difference)."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import test_host
    from conftest import load_golden
    dref, _ = load_golden(name)
    inp = test_host._make_golden().inputs_for(name)
    rec = inp.receptor
    xyz, ic = evaluator.cleft_grid(rec.cleft_center, [rec.cleft_radius], 0.375, dref.ori)
    full = synth.cleft_grid(rec.cleft_center, rec.cleft_radius, 0.375)
    np.testing.assert_array_equal(xyz, full)
    # the fixture keeps a subset of the grid (make_golden.py); find each of its points
    g = np.asarray(inp.grid_xyz, np.float32)
    idx = {tuple(p): i for i, p in enumerate(map(tuple, xyz))}
    rows = np.array([idx[tuple(p)] for p in map(tuple, g)])
    ref = np.asarray(dref.grid_ic[1:], np.float32)
    ulps = np.abs(ic[rows].view(np.int32).astype(np.int64) - ref.view(np.int32).astype(np.int64))
    print(f"{name}: {len(rows)} grid points, {(ulps > 0).any(axis=1).sum()} differ from the reference in the "
          f"last place (at most {ulps.max()} units)")
    assert ulps.max() <= 2


def test_cell_list_on_device_keeps_parity(tiny_system):
    """Contexts build their cell list on the device; the tiny system's poses match the oracle."""
    from oracle import port
    _, d = tiny_system
    genes = synth.random_genes(512, d.n_genes, seed=9)
    ev = evaluator.GPUEvaluator(d, max_poses=512)
    g = ev.eval_genes(genes)
    port.set_reference_compat(True)
    r = port.Oracle(d).eval_ic(d.genes_to_ic(genes))["cf"]
    np.testing.assert_array_equal(g["status"], r["status"])
    ok = g["status"] == 0
    assert ok.sum() > 10
    assert (np.abs(g["evalue"][ok] - r["evalue"][ok]) / np.maximum(1.0, np.abs(r["evalue"][ok]))).max() <= 1e-9
    ev.close()
