"""Generates the golden fixtures of the CF-based clustering from the reference itself.

Run from the repository root in a checkout that has the reference sources and the compiled
reference (``make -C oracle ref``, which compiles LIB/cluster.cpp, calc_rmsd_chrom.cpp and
write_pdb.cpp together with the scoring chain):

    python tests/golden/make_golden_cluster.py

For each system it writes ``tests/golden/cluster_<name>.npz`` holding the descriptor exported by
the reference's own set-up (cleft grid cut to its first points so the fixture stays small), a
seeded ensemble with structure to cluster (``synth.clustered_ensemble``: chromosomes a few bins
around random centres, sorted by energy), and, for each clustering case (temperature,
cluster_rmsd, max_results), the text of the .cad file the reference's cluster() wrote, and for the
first case the PDB file of its first result (write_pdb) with the ligand's bond list.
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from flexaidds_gb300 import synth, system  # noqa: E402
from oracle import ref  # noqa: E402  (used only when run as a script)

OUT = os.path.dirname(os.path.abspath(__file__))

# (receptor atoms, cleft radius, ligand atoms, torsions, seed, side chains, grid points kept,
#  centres, variants per centre)
SYSTEMS = {
    "flex_900_16": (900, 7.0, 16, 4, 45, 2, 3000, 12, 40),
    "lig_2000_24": (2000, 8.0, 24, 6, 11, 0, 3000, 20, 30),
}
# (temperature K, cluster_rmsd, max_results): the reference's defaults (0, 2.0, 10), Boltzmann-
# weighted terms with the ACF sort, more entries than clusters (zero entries sorted in), and
# many small clusters
CASES = [(0, 2.0, 10), (300, 2.0, 10), (300, 2.0, 80), (0, 1.0, 150), (310, 3.0, 25)]


def make(name):
    n_rec, rad, n_lig, n_tor, seed, sc, n_grid, centres, per = SYSTEMS[name]
    inp = system.make_inputs(n_rec, rad, n_lig, n_tor, seed=seed, side_chains=sc)
    inp.grid_xyz = np.ascontiguousarray(inp.grid_xyz[:n_grid])
    h = ref.RefHarness(inp)
    d = h.descriptor()
    ic, e = synth.clustered_ensemble(d, centres, per, seed=seed + 7)
    arrs = d.to_arrays("d_")
    arrs.update(ic=ic, app_evalue=e, cases=np.asarray(CASES, np.float64))
    arrs["lig_bonds"] = np.asarray(inp.ligand.bonds, np.int32).reshape(-1, 2)
    with tempfile.TemporaryDirectory() as tmp:
        for k, (T, thr, R) in enumerate(CASES):
            txt = h.cluster(ic, e, int(T), float(thr), int(R), os.path.join(tmp, f"case{k}"))
            arrs[f"cad_{k}"] = np.frombuffer(txt.encode(), np.uint8)
            if k == 0:
                # the pose file of the first result (write_pdb after ic2cf of its head)
                with open(os.path.join(tmp, "case0_0.pdb"), "rb") as f:
                    arrs["pdb_0"] = np.frombuffer(f.read(), np.uint8)
    path = os.path.join(OUT, f"cluster_{name}.npz")
    np.savez_compressed(path, **arrs)
    print(f"{path}: {ic.shape[0]} chromosomes, {len(CASES)} cases, {os.path.getsize(path) / 1024:.0f} KB")


if __name__ == "__main__":
    if not ref.available():
        sys.exit("the compiled reference is missing: run make -C oracle ref")
    names = sys.argv[1:]
    if names:
        for name in names:
            make(name)
    else:
        # the reference keeps its state in globals: one process per system
        import subprocess
        for name in SYSTEMS:
            subprocess.run([sys.executable, os.path.abspath(__file__), name], check=True)
