"""Times the C restatement (oracle/fxe_oracle.c, the CPU baseline of bench.py) against the
reference's own scoring chain compiled from its sources (oracle/_ref/libfxe_ref.so) on the same
poses of the benchmark's system, one core each, and checks that both give the same records.

TEST INFRASTRUCTURE ONLY. Needs the compiled reference (``make -C oracle ref`` in a checkout with
the reference sources); run from the repository root:

    python oracle/calibrate_port.py [n_poses]

The system is the benchmark's (6,000-atom receptor with three flexible side chains of eight
rotamers, 48-atom ligand, 12 torsions; its full cleft grid), set up by the reference itself
(RefHarness.descriptor); the poses are the first n_poses (default 2,000) uniform chromosomes that
pass the clash pre-filter, as the benchmark's populations are.
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from flexaidds_gb300 import synth, system  # noqa: E402
from oracle import port, ref  # noqa: E402

WORKLOAD = dict(n_rec=6000, cleft=12.0, n_lig=48, n_tor=12, seed=7, edge=60.032427451306646,
                side_chains=3, rotamers=8)


def main(n_poses: int = 2000):
    if not ref.available():
        sys.exit("the compiled reference scoring chain is missing: run make -C oracle ref")
    w = WORKLOAD
    inp = system.make_inputs(w["n_rec"], w["cleft"], w["n_lig"], w["n_tor"], seed=w["seed"], edge=w["edge"],
                             side_chains=w["side_chains"], rotamers=w["rotamers"])
    h = ref.RefHarness(inp)
    d = h.descriptor()
    port.set_reference_compat(True)
    port.set_trig_rounding(False)
    o = port.Oracle(d)
    # the first n_poses uniform chromosomes that pass the clash pre-filter
    keep, k = [], 0
    while sum(len(x) for x in keep) < n_poses:
        g = synth.random_genes(20_000, d.n_genes, seed=w["seed"] * 1000 + k)
        ic = d.genes_to_ic(g)
        keep.append(ic[o.eval_ic(ic)["cf"]["status"] == 0])
        k += 1
    ic = np.ascontiguousarray(np.concatenate(keep)[:n_poses])

    # alternating runs, the best of three each (the host's other load varies)
    t_ref = t_port = float("inf")
    for _ in range(3):
        t0 = time.perf_counter()
        cf_ref, st_ref, _ = h.eval(ic)
        t1 = time.perf_counter()
        r = o.eval_ic(ic)["cf"]
        t2 = time.perf_counter()
        t_ref, t_port = min(t_ref, t1 - t0), min(t_port, t2 - t1)
    same_status = bool(np.array_equal(r["status"], st_ref))
    ok = st_ref == 0
    # (the harness's records: the cfstr terms, the CF in column 9, rclash in column 10)
    rel = np.abs(r["evalue"][ok] - cf_ref[ok, 9]) / np.maximum(1.0, np.abs(cf_ref[ok, 9]))
    print(f"{n_poses} scored poses of the benchmark system on one core of {os.uname().machine}:")
    print(f"  compiled reference (ic2cf from its own sources): {n_poses / t_ref:,.0f} poses/s ({t_ref:.2f} s)")
    print(f"  C restatement (bench.py's CPU baseline):        {n_poses / t_port:,.0f} poses/s ({t_port:.2f} s)")
    print(f"  ratio restatement / reference: {t_ref / t_port:.3f}")
    print(f"  statuses identical: {same_status}; CF: {int((rel == 0).sum())} of {int(ok.sum())} identical, "
          f"largest relative difference {rel.max():.1e}")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 2000)
