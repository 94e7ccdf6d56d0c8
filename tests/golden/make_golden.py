"""Generates the golden fixtures of the fitness-evaluation path from the reference itself.

Run from the repository root in a checkout that has the reference sources and the compiled
reference scoring chain (``make -C oracle ref``):

    python tests/golden/make_golden.py

For each system it writes ``tests/golden/<name>.npz`` holding
  * the descriptor exported by the reference's own set-up (buildic, buildlist, assign_shift,
    bonded lists, calc_cleftic, ic_bounds, add2_optimiz_vec), with the cleft grid subsampled so
    the fixture stays small;
  * int32 chromosomes and their decoded ICs (genetoic restated; the reference's decoder lives in
    LIB/gaboom.cpp, which does not compile without Eigen);
  * what the reference's ic2cf returns for every chromosome (the 11 cfstr terms and the status
    class), the ligand coordinates buildcc produced, and, for the first poses, the contact lists
    (partner Calc index, area) Vcontacts recorded per scored atom (side-chain atoms, then the
    ligand).

Chromosomes are drawn uniformly, then filtered with the C restatement so that the fixture holds
mostly poses that get scored (uniform chromosomes clash about nine times in ten), some clashes
and every polyhedron failure met on the way.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from flexaidds_gb300 import synth, system  # noqa: E402
from oracle import port, ref  # noqa: E402  (used only when run as a script)

OUT = os.path.dirname(os.path.abspath(__file__))


def density_curves(inp, seed, frac=0.3):
    """Turns a fraction of the energy-matrix pairs into piecewise-linear density curves."""
    rng = np.random.default_rng(seed)
    t = inp.emat.shape[0]
    w = np.ones((t, t), np.int32)
    curves = {}
    for i in range(t):
        for j in range(i, t):
            if rng.random() < frac:
                w[i, j] = w[j, i] = 0
                xs = np.sort(rng.uniform(0.0, 1.0, size=int(rng.integers(2, 5))))
                xs[0] = 0.0
                ys = rng.normal(size=xs.size)
                curves[(i, j)] = [(float(x), float(y)) for x, y in zip(xs, ys)]
    inp.emat_weight = w
    inp.emat_curves = curves


SYSTEMS = {
    # 2,000-atom receptor, 8 A cleft, 24-atom ligand with 6 torsions, single-value matrix
    "c0_2000_24": dict(args=(2000, 8.0, 24, 6), seed=11, grid=1024, pool=6000, scored=160,
                       clashed=40, contacts=16, tweak=None),
    # 900-atom receptor, 7 A cleft, 16-atom ligand, 4 torsions, density curves, other switches
    "curves_900_16": dict(args=(900, 7.0, 16, 4), seed=23, grid=512, pool=4000, scored=100,
                          clashed=20, contacts=8, tweak="curves"),
    # 600-atom receptor, 6 A cleft, 10-atom ligand; half the grid points lie outside the
    # receptor's box, so poses leave it: index_protein re-derives its cell grid for them, and
    # atoms without contacts take the SAS-only path
    "outside_600_10": dict(args=(600, 6.0, 10, 2), seed=37, grid=256, pool=3000, scored=120,
                           clashed=20, contacts=8, tweak="outside"),
    # the at-scale shape of the benchmark: 6,000-atom receptor, 12 A cleft, 48-atom ligand with
    # 12 torsions (receptor cube edge given, as the benchmark gives it)
    "scale_6000_48": dict(args=(6000, 12.0, 48, 12), seed=7, grid=768, pool=40000, scored=60,
                          clashed=10, contacts=3, tweak=None, edge=60.032427451306646),
    # flexible side chains: three residues of eight rotamers carved into the cleft wall, their
    # rotamer genes last
    "flex_2000_24": dict(args=(2000, 8.0, 24, 6), seed=11, grid=1024, pool=8000, scored=120,
                         clashed=30, contacts=8, tweak=None, side_chains=3),
    # side chains with density curves, the other switches and intramolecular terms off
    "flexcurves_900_16": dict(args=(900, 7.0, 16, 4), seed=23, grid=512, pool=6000, scored=80,
                              clashed=20, contacts=6, tweak="curves", side_chains=2, intramolecular=0),
    # the benchmark's shape with its three side chains
    "flexscale_6000_48": dict(args=(6000, 12.0, 48, 12), seed=7, grid=768, pool=60000, scored=50,
                              clashed=10, contacts=2, tweak=None, edge=60.032427451306646,
                              side_chains=3),
}


def inputs_for(name):
    """The generator inputs of fixture ``name`` (seeded; the cleft grid subsampled)."""
    cfg = SYSTEMS[name]
    n_rec, cleft, n_lig, n_tor = cfg["args"]
    inp = system.make_inputs(n_rec, cleft, n_lig, n_tor, seed=cfg["seed"], edge=cfg.get("edge"),
                             side_chains=cfg.get("side_chains", 0))
    inp.intramolecular = cfg.get("intramolecular", 1)
    rng = np.random.default_rng(cfg["seed"] + 100)
    keep = np.sort(rng.choice(inp.grid_xyz.shape[0], cfg["grid"], replace=False))
    inp.grid_xyz = np.ascontiguousarray(inp.grid_xyz[keep])
    if cfg["tweak"] == "outside":
        # replace half of the grid with points 1-6 A beyond the faces of the receptor's box
        lo, hi = inp.receptor.xyz.min(axis=0), inp.receptor.xyz.max(axis=0)
        m = inp.grid_xyz.shape[0] // 2
        pts = rng.uniform(lo, hi, size=(m, 3))
        axis = rng.integers(0, 3, size=m)
        side = rng.integers(0, 2, size=m)
        off = rng.uniform(1.0, 6.0, size=m)
        for k in range(m):
            a = axis[k]
            pts[k, a] = hi[a] + off[k] if side[k] else lo[a] - off[k]
        inp.grid_xyz = np.ascontiguousarray(np.concatenate([inp.grid_xyz[m:], pts]).astype(np.float32))
    if cfg["tweak"] == "curves":
        density_curves(inp, cfg["seed"] + 200)
        inp.permeability = 0.9
        inp.dee_clash = 0.6
        inp.solventterm = 0.35
    return inp


def make(name, cfg):
    inp = inputs_for(name)
    h = ref.RefHarness(inp)
    d = h.descriptor()

    genes = synth.random_genes(cfg["pool"], d.n_genes, seed=cfg["seed"] + 300)
    ic = d.genes_to_ic(genes)
    port.set_reference_compat(True)
    port.set_trig_rounding(False)
    st = port.Oracle(d).eval_ic(ic)["cf"]["status"]
    sel = np.concatenate([np.nonzero(st == 0)[0][:cfg["scored"]], np.nonzero(st == 2)[0][:cfg["clashed"]],
                          np.nonzero(st == 1)[0]])
    sel = np.sort(sel)
    genes, ic = genes[sel], ic[sel]

    cf, status, xyz = h.eval(ic, want_xyz=True)
    # contact lists of the first scored poses, one pose per call
    cpose = np.nonzero(status == 0)[0][:cfg["contacts"]]
    c_pose, c_atom, c_part, c_area = [], [], [], []
    for p in cpose:
        h.eval(ic[p:p + 1])
        for a, (part, area, _dist) in enumerate(h.last_contacts()):
            c_pose += [p] * len(part)
            c_atom += [a] * len(part)
            c_part += list(part)
            c_area += list(area)
    arrs = d.to_arrays("d_")
    arrs.update(genes=genes, ic=ic, cf=cf, status=status, xyz=xyz,
                c_pose=np.asarray(c_pose, np.int32), c_atom=np.asarray(c_atom, np.int32),
                c_partner=np.asarray(c_part, np.int32), c_area=np.asarray(c_area, np.float64))
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **arrs)
    print(f"{path}: {len(sel)} poses ({(status == 0).sum()} scored, {(status == 2).sum()} clashed, "
          f"{(status == 1).sum()} polyhedron failures), {len(c_pose)} contacts, "
          f"{os.path.getsize(path) / 1024:.0f} KB")


if __name__ == "__main__":
    if not ref.available():
        sys.exit("the compiled reference scoring chain is missing: run make -C oracle ref")
    names = sys.argv[1:]
    if names:
        for name in names:
            make(name, SYSTEMS[name])
    else:
        # the reference keeps its scoring state in globals: one process per system
        import subprocess
        for name in SYSTEMS:
            subprocess.run([sys.executable, os.path.abspath(__file__), name], check=True)
