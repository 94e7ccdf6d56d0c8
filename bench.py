"""Throughput of the GA fitness-evaluation path on GB300: poses scored per second.

A step is one GA generation's evaluation: one population of 2,000 chromosomes scored in one
launch sequence (decode -> build -> contact candidates -> Voronoi polyhedra -> complementarity
score). The workload is the plain, one-job-per-launch configuration at scale: a 6,000-atom
seeded Poisson-disc receptor (12 A cleft, 0.375 A grid of 137,060 points), a 48-atom ligand with
12 torsions, 40 atom types, a 40 x 40 N(0,1) energy matrix. Every chromosome of a population
passes the clash pre-filter, so every pose goes through the polyhedron and scoring stages (the
populations are the first chromosomes of a seeded uniform stream that do; uniform chromosomes
clash about 99 times in 100 on this system and cost far less).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision reference|fast]
  python bench.py --impl reference ...   the same workload on the host cores (CPU restatement)
  python bench.py --cluster-only C       only the clustering of C x 500 chromosomes (profiling)

Beside the headline, the JSON line carries the statmech reduction of 1e6 energies, the batched
many-ligand workload, the served Poisson streams and the clustering of a 1e6-chromosome ensemble
(each leg can be switched off: --batched 0, --served 0, --cluster 0).

Several GPUs run independent replicas (the path has no exchange step); value counts all ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from flexaidds_gb300 import capi, prepare, synth, system  # noqa: E402

METRIC = "poses scored/s on 1 GB300 (plain path, one population per launch)"
WORKLOAD = dict(n_rec=6000, cleft=12.0, n_lig=48, n_tor=12, seed=7, edge=60.032427451306646,
                population=2000, side_chains=3, rotamers=8)
WORKLOAD_NAME = ("plain-scale: 6000-atom receptor (before carving the side chains), 12 A cleft "
                 "(137060 grid points), 48-atom ligand, 12 torsions, 3 flexible side chains of 8 "
                 "rotamers (19 genes), populations of 2000 chromosomes that all pass the clash "
                 "pre-filter")
N_POPULATIONS = 8           # distinct populations, cycled over the steps
FLUSH_BYTES = 512 << 20     # L2 flush between timed steps (L2 is 129 MB)
STATMECH_N = 1_000_000      # ensemble size of the thermodynamics reduction (all poses of a run)

# DRAM bytes per launch of the dominant kernel from ncu (dram__bytes_read.sum +
# dram__bytes_write.sum), keyed by precision; from profiles/pose_kernel_plain_scale.md.
POSE_KERNEL_DRAM_BYTES = {"reference": 102_597_888, "fast": 85_202_176}

# nominal non-tensor arithmetic peaks of GB300 (152 SMs at 2,070 MHz): FP32 152 x 128 lanes x 2
# flops per FMA; FP64 1.25 TFLOP/s. There is no measured figure for either.
NOMINAL_PEAK_TFLOPS = {"fast": 152 * 128 * 2 * 2.07e9 / 1e12, "reference": 1.25}


def work_flops_per_pose(c: dict) -> float:
    """Algorithmic work of one pose from the oracle's per-pose mean counts:
    sum over scored atoms (ligand and side-chain atoms) of 8 C + 14 NC + 12 NC E + 60 E_arc +
    40 T + 30 V, plus 60 per built
    atom (C candidates scanned, NC contacts, E hull edges, E_arc arc edges, T spherical triangles
    and arc segments, V vertices)."""
    return (8 * c["candidates"] + 14 * c["contacts"] + 12 * c["plane_tests"] + 60 * c["arc_edges"]
            + 40 * c["triangles"] + 30 * c["vertices"] + 60 * c["built_atoms"])


# ---------------------------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------------------------

def make_system():
    w = WORKLOAD
    inp = system.make_inputs(w["n_rec"], w["cleft"], w["n_lig"], w["n_tor"], seed=w["seed"],
                             edge=w["edge"], side_chains=w["side_chains"], rotamers=w["rotamers"])
    return prepare.prepare(inp)


def uniform_block(d, k):
    """Block k of the seeded uniform chromosome stream (100,000 chromosomes)."""
    return synth.random_genes(100_000, d.n_genes, seed=WORKLOAD["seed"] * 1000 + k)


def scored_populations(d, n_pop, status_of):
    """The first n_pop * population chromosomes of the uniform stream that pass the clash
    pre-filter; status_of(genes) -> pose status per chromosome."""
    need = n_pop * WORKLOAD["population"]
    keep, k = [], 0
    while sum(len(x) for x in keep) < need:
        g = uniform_block(d, k)
        keep.append(g[status_of(g) == capi.POSE_SCORED])
        k += 1
        if k > 2000:
            raise RuntimeError("too few chromosomes pass the clash pre-filter")
    allg = np.concatenate(keep)[:need]
    return allg.reshape(n_pop, WORKLOAD["population"], d.n_genes)


# ---------------------------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path:
            return None
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------------------

def cpu_baseline_port(d, pops, seconds=10.0):
    """The CPU restatement on one host core over whole populations, about `seconds` of work."""
    from oracle import port
    o = port.Oracle(d)
    ic = d.genes_to_ic(pops[0])
    n, t0 = 0, time.perf_counter()
    while True:
        o.eval_ic(ic)
        n += ic.shape[0]
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "poses/s", "cores": 1, "kind": "port",
            "sample": f"{n} poses ({n // ic.shape[0]} passes over one population of "
                      f"{ic.shape[0]}), {dt:.1f} s on 1 core of {cpu_model()}"}


def oracle_counts(d, genes):
    from oracle import port
    r = port.Oracle(d).eval_ic(d.genes_to_ic(genes), counts=True)
    n = genes.shape[0]
    return {k: v / n for k, v in r["counts"].items()}


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
        return f"{os.uname().machine} ({os.cpu_count()} cores)"
    except OSError:
        return "unknown"


class Ranks:
    """Replicas, one process per GPU (torchrun sets RANK / WORLD_SIZE / MASTER_*): a barrier and
    the maximum of a value over ranks. A single process when WORLD_SIZE is unset."""

    def __init__(self, backend: str, device: str):
        import torch
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.device = device
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend)
            self.dist = dist
        self._torch = torch

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()
        if self.device.startswith("cuda"):
            self._torch.cuda.synchronize()

    def max(self, x: float) -> float:
        if self.dist is None:
            return x
        t = self._torch.tensor([x], dtype=self._torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()


def run_gpu(args):
    import torch
    from flexaidds_gb300 import evaluator

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    ranks = Ranks("nccl", "cuda")
    world, rank = ranks.world, ranks.rank
    barrier, max_over_ranks = ranks.barrier, ranks.max

    prec = args.precision
    d = make_system()
    pop = WORKLOAD["population"]
    ev = evaluator.GPUEvaluator(d, max_poses=pop,
                                precision=0 if prec == "reference" else 1)
    filt = evaluator.GPUEvaluator(d, max_poses=100_000, precision=1)
    pops = scored_populations(d, N_POPULATIONS, lambda g: filt.eval_genes(g)["status"])
    filt.close()

    stream = torch.cuda.Stream()
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    dgen = [torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in pops]
    dout = torch.empty(pop * capi.CF_DTYPE.itemsize, dtype=torch.uint8, device="cuda")

    def step(k):
        ev.eval_genes_device(dgen[k % N_POPULATIONS].data_ptr(), pop, dout.data_ptr(), stream.cuda_stream)

    # --- device-resident: inputs in HBM, timed on the launching stream -----------------------
    with torch.cuda.stream(stream):
        for k in range(args.warmup):
            flush.zero_()
            step(k)
    stream.synchronize()
    ev.enable_timing(True)
    ev.take_timing()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        torch.cuda.nvtx.range_push("timed")   # profilers select the timed launches by this range
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                starts[k].record(stream)
                step(args.warmup + k)
                ends[k].record(stream)
        stream.synchronize()
        torch.cuda.nvtx.range_pop()
        barrier()
        wall = time.perf_counter() - t0
    stage_ms, launches = ev.take_timing()
    ev.enable_timing(False)
    dev_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    dev_ms = max_over_ranks(dev_ms)
    value = world * pop * args.steps / (dev_ms / 1e3)

    # --- end to end: host buffers through the C ABI, copies inside the timed region ----------
    lib = evaluator.load_library()
    hgen = [torch.from_numpy(np.ascontiguousarray(p)).pin_memory() for p in pops]
    hout = torch.empty(pop * capi.CF_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
    for k in range(args.warmup):
        lib.fxe_eval_genes(ev.handle, pop, C.cast(hgen[k % N_POPULATIONS].data_ptr(), capi._i),
                           C.c_void_p(hout.data_ptr()))
    e2e_s = 0.0
    barrier()
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        rc = lib.fxe_eval_genes(ev.handle, pop, C.cast(hgen[k % N_POPULATIONS].data_ptr(), capi._i),
                                C.c_void_p(hout.data_ptr()))
        e2e_s += time.perf_counter() - t
        if rc != 0:
            raise RuntimeError(lib.fxe_last_error().decode())
    barrier()
    e2e_s = max_over_ranks(e2e_s)
    res = np.frombuffer(hout.numpy().tobytes(), capi.CF_DTYPE)
    assert np.all(res["status"] != capi.POSE_CAPACITY)

    # --- statmech over a run's ensemble (1e6 poses, FP64) -------------------------------------
    from flexaidds_gb300.capi import Thermo
    energies = torch.from_numpy(np.random.default_rng(1).normal(-30.0, 5.0, STATMECH_N)).cuda()
    th = Thermo()
    for _ in range(3):
        lib.fxe_thermo_compute_device(C.c_void_p(energies.data_ptr()), None, STATMECH_N, 300.0,
                                      C.byref(th), C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    sm_ms = []
    for _ in range(10):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        lib.fxe_thermo_compute_device(C.c_void_p(energies.data_ptr()), None, STATMECH_N, 300.0,
                                      C.byref(th), C.c_void_p(stream.cuda_stream))
        b.record(stream)
        b.synchronize()
        sm_ms.append(a.elapsed_time(b))
    sm_best = min(sm_ms)

    clustered = run_cluster(ev, d) if args.cluster else None
    batched = run_batched(args, prec, flush, stream) if args.batched else None
    served = None
    if args.served:
        from flexaidds_gb300.system import SystemInputs  # noqa: F401
        w, b = WORKLOAD, BATCH
        served = run_served(prec, {
            "6000": system.make_inputs(w["n_rec"], w["cleft"], 12, 3, seed=w["seed"], edge=w["edge"],
                                       side_chains=w["side_chains"], rotamers=w["rotamers"]),
            "4000": system.make_inputs(b["n_rec"], b["cleft"], 12, 3, seed=b["seed"], edge=b["edge"])})

    if rank != 0:
        ranks.close()
        return

    # --- roofline of the dominant kernel (polyhedra + scoring) --------------------------------
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    counts = oracle_counts(d, pops[0][:256])
    flop_pose = work_flops_per_pose(counts)
    pose_ms = stage_ms[2] / args.steps
    achieved = flop_pose * pop / (pose_ms / 1e3) / 1e12
    peak = NOMINAL_PEAK_TFLOPS[prec]
    traffic = POSE_KERNEL_DRAM_BYTES[prec]
    hbm = peaks.get("hbm_gbs")
    sm_gbs = 8.0 * STATMECH_N / (sm_best / 1e3) / 1e9
    try:
        cpu = cpu_baseline_port(d, pops)
    except Exception as e:   # the oracle library could not be built or loaded
        cpu = {"value": None, "unit": "poses/s", "cores": 1, "kind": "port", "sample": f"unavailable: {e}"}

    out = {
        "metric": METRIC, "value": value, "unit": "poses/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == "reference" else "f32",
        "data": "synthetic (seeded Poisson-disc receptor, seeded tree ligand, N(0,1) matrix)",
        "config": {"workload": WORKLOAD_NAME, "population": pop, "precision": prec,
                   "l2": f"flushed between timed steps ({FLUSH_BYTES >> 20} MB write)",
                   "parallelism": f"replicas x{world}",
                   "side_chains": f"{d.n_flex} residues x {int(d.flex_nrot[0]) if d.n_flex else 0} "
                                  f"rotamers, {d.n_sc} scored side-chain atoms"},
        "e2e": {"value": world * pop * args.steps / e2e_s, "unit": "poses/s",
                "h2d_bytes_per_step": pop * d.n_genes * 4, "d2h_bytes_per_step": pop * capi.CF_DTYPE.itemsize},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "roofline": {"bound": "fp64" if prec == "reference" else "fp32", "achieved": achieved,
                     "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "nominal (no measured non-tensor peak)",
                     "kernel": f"pose_kernel ({prec})", "flop_per_pose": flop_pose,
                     "launch_ms": pose_ms},
        "cpu_baseline": cpu,
        "stage_ms_per_step": {"build": stage_ms[0] / args.steps, "candidates": stage_ms[1] / args.steps,
                              "polyhedra_and_scoring": pose_ms},
        "wall_s_timed_region": wall,
        "statmech": {"poses": STATMECH_N, "ms": sm_best, "poses_per_s": STATMECH_N / (sm_best / 1e3),
                     "roofline": {"bound": "hbm", "achieved": sm_gbs, "peak": hbm, "unit": "GB/s",
                                  "frac": (sm_gbs / hbm) if hbm else None, "traffic": None}},
        "batched": batched,
        "served": served,
        "cluster": clustered,
    }
    print(json.dumps(out), flush=True)
    ranks.close()


# ---------------------------------------------------------------------------------------------
# clustering of a run's ensemble (cluster, LIB/cluster.cpp): 1e6 chromosomes, the reference's
# default options (cluster_rmsd 2.0, max_results 10, temperature 0)
# ---------------------------------------------------------------------------------------------

CLUSTER = dict(centres=2000, per_centre=500, seed=17, rmsd=2.0, max_results=10, temperature=0,
               cpu_sample=20_000)


def run_cluster(ev, d, centres=None):
    """Device time of fxe_cluster's kernels (CUDA events inside the call), its end-to-end time
    (host ICs and energies in, results out), and the C restatement on a bounded sample."""
    c = dict(CLUSTER)
    if centres:
        c["centres"] = centres
    ic, e = synth.clustered_ensemble(d, c["centres"], c["per_centre"], seed=c["seed"])
    n = ic.shape[0]
    args = (ic, e, c["temperature"], c["rmsd"], c["max_results"])
    ev.cluster(*args)                                       # warm-up
    dev, e2e = [], []
    for _ in range(3):
        t = time.perf_counter()
        r = ev.cluster(*args)
        e2e.append(time.perf_counter() - t)
        dev.append(ev.cluster_time())
    out = {"workload": f"{n} chromosomes of the plain-scale system ({c['centres']} centres x "
                       f"{c['per_centre']} variants a few bins apart, sorted by energy), "
                       f"cluster_rmsd {c['rmsd']}, max_results {c['max_results']}, "
                       f"temperature {c['temperature']}",
           "clusters": int(r["n_clusters"]), "clustered": int(r["freq"].sum()),
           "device_ms": min(dev), "e2e_ms": 1e3 * min(e2e),
           "chromosomes_per_s": n / (min(dev) / 1e3), "e2e_chromosomes_per_s": n / min(e2e),
           "kernels_per_call": 2 + c["max_results"] + (1 if c["temperature"] else 0)}
    try:
        from oracle import port
        m = c["cpu_sample"]
        o = port.Oracle(d)
        t = time.perf_counter()
        o.cluster(ic[:m], e[:m], c["temperature"], c["rmsd"], c["max_results"])
        cs = time.perf_counter() - t
        out["cpu_baseline"] = {"value": m / cs, "unit": "chromosomes/s", "cores": 1, "kind": "port",
                               "sample": f"first {m} chromosomes of the same ensemble"}
    except Exception as ex:   # the oracle library could not be built or loaded
        out["cpu_baseline"] = {"value": None, "sample": f"unavailable: {ex}"}
    return out


# ---------------------------------------------------------------------------------------------
# batched: many ligands on one receptor, one launch per generation
# ---------------------------------------------------------------------------------------------

BATCH = dict(n_rec=4000, cleft=10.0, seed=31, edge=51.92391670510951, jobs=256, atoms=(10, 70),
             torsions=(0, 15), population=(200, 2000))
BATCH_NAME = ("batched: 4000-atom receptor, 10 A cleft (79501 grid points), 256 seeded ligands of "
              "U[10,70] heavy atoms and U[0,15] torsions, populations U[200,2000] of uniform "
              "(initial-generation) chromosomes; one GA generation of every job per step")


def make_batch_jobs():
    from flexaidds_gb300.system import SystemInputs
    b = BATCH
    base = system.make_inputs(b["n_rec"], b["cleft"], 12, 3, seed=b["seed"], edge=b["edge"])
    rng = np.random.default_rng(b["seed"] + 1)
    out = []
    for k in range(b["jobs"]):
        n = int(rng.integers(b["atoms"][0], b["atoms"][1] + 1))
        t = int(rng.integers(b["torsions"][0], b["torsions"][1] + 1))
        pop = int(rng.integers(b["population"][0], b["population"][1] + 1))
        lig = synth.random_ligand(n, t, seed=b["seed"] * 1000 + k)
        d = prepare.prepare(SystemInputs(receptor=base.receptor, ligand=lig, grid_xyz=base.grid_xyz,
                                         emat=base.emat))
        out.append((d, pop, synth.random_genes(pop, d.n_genes, seed=b["seed"] * 5000 + k)))
    return out


def run_batched(args, prec, flush, stream):
    """Poses/s of one generation of all jobs: one launch sequence per job (the plain path) and
    one batched launch for all of them, same chromosomes, device-resident, L2 flushed."""
    import torch
    from flexaidds_gb300 import evaluator
    jobs = make_batch_jobs()
    p = 0 if prec == "reference" else 1
    first = evaluator.GPUEvaluator(jobs[0][0], max_poses=jobs[0][1], precision=p)
    evs = [first] + [evaluator.GPUEvaluator(d, max_poses=pop, precision=p, share_receptor_with=first)
                     for d, pop, _ in jobs[1:]]
    dg = [torch.from_numpy(np.ascontiguousarray(g)).cuda() for _, _, g in jobs]
    do = [torch.empty(pop * capi.CF_DTYPE.itemsize, dtype=torch.uint8, device="cuda") for _, pop, _ in jobs]
    total = sum(pop for _, pop, _ in jobs)
    batch = evaluator.Batch(max_jobs=len(jobs), max_poses=total, max_genes=64)
    table = [(ev, pop, g.data_ptr(), o.data_ptr()) for ev, (_, pop, _), g, o in zip(evs, jobs, dg, do)]

    def plain():
        for ev, pop, g, o in table:
            ev.eval_genes_device(g, pop, o, stream.cuda_stream)

    def batched():
        batch.eval_genes_device(table, stream.cuda_stream)

    res = {}
    steps = max(1, min(args.steps, 5))
    for name, fn in (("plain", plain), ("batched", batched)):
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                fn()
        stream.synchronize()
        ms = 0.0
        for _ in range(steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                a.record(stream)
                fn()
                b.record(stream)
            b.synchronize()
            ms += a.elapsed_time(b)
        res[name] = {"poses_per_s": total * steps / (ms / 1e3), "ms_per_generation": ms / steps}
    batched_out = [np.frombuffer(o.cpu().numpy().tobytes(), capi.CF_DTYPE) for o in do]
    plain()
    stream.synchronize()
    plain_out = [np.frombuffer(o.cpu().numpy().tobytes(), capi.CF_DTYPE) for o in do]
    same = all(np.array_equal(a, b) for a, b in zip(batched_out, plain_out))
    scored = sum(int((o["status"] == capi.POSE_SCORED).sum()) for o in plain_out)
    for ev in evs:
        ev.close()
    batch.close()
    return {"workload": BATCH_NAME, "jobs": len(jobs), "poses_per_generation": total,
            "scored_fraction": scored / total, "precision": prec, "steps": steps,
            "plain": res["plain"], "batched": res["batched"],
            "speedup": res["batched"]["poses_per_s"] / res["plain"]["poses_per_s"],
            "results_identical": same}


# ---------------------------------------------------------------------------------------------
# served: Poisson arrivals of docking jobs, continuous batching on the device GA engine
# ---------------------------------------------------------------------------------------------

SERVE = dict(rates=(10.0, 50.0, 200.0), jobs=48, population=500, generations=20, budget=150e9,
             atoms_median=30, atoms=(10, 70), torsions=(0, 15), seed=77)
SERVE_NAME = ("served: Poisson arrivals at 10, 50 and 200 jobs/s, 48 jobs per rate, receptors from a "
              "cache of two (6000 atoms with three flexible side chains of 8 rotamers, and 4000 "
              "atoms), ligands lognormal median 30 heavy atoms (10-70) with U[0,15] torsions, "
              "population 500 for 20 generations, the reference's GA defaults (PSHARE fitness, "
              "BOOM, duplicates rejected), 150 GB admission budget")


def run_served(prec, receptors):
    from flexaidds_gb300 import serve
    from flexaidds_gb300.system import SystemInputs
    s = SERVE
    rng = np.random.default_rng(s["seed"])
    reqs = []
    keys = list(receptors)
    for k in range(s["jobs"]):
        key = keys[k % len(keys)]
        base = receptors[key]
        n = int(np.clip(round(rng.lognormal(np.log(s["atoms_median"]), 0.4)), *s["atoms"]))
        t = int(rng.integers(s["torsions"][0], s["torsions"][1] + 1))
        lig = synth.random_ligand(n, t, seed=s["seed"] * 1000 + k)
        d = prepare.prepare(SystemInputs(receptor=base.receptor, ligand=lig, grid_xyz=base.grid_xyz, emat=base.emat))
        reqs.append(serve.JobRequest(0.0, key, d, s["population"], s["generations"], seed=s["seed"] * 7919 + k))
    p = 0 if prec == "reference" else 1
    out = {"workload": SERVE_NAME, "precision": prec, "rates": []}
    for rate in s["rates"]:
        arr = serve.poisson_arrivals(len(reqs), rate, seed=int(rate))
        for r, t in zip(reqs, arr):
            r.arrival = float(t)
        srv = serve.DockingServer(max_jobs=256, hbm_budget=s["budget"], precision=p)
        res = srv.run(reqs)
        launches, graphs = srv.engine.take_launches()
        srv.close()
        summ = serve.latency_summary(res)
        poses = len(res) * s["population"] * (s["generations"] + 1)
        summ.update({"arrival_rate": rate, "poses_per_s": poses / summ["makespan_s"],
                     "graph_launches": graphs, "kernel_launches": launches})
        out["rates"].append(summ)
    return out


# ---------------------------------------------------------------------------------------------
# reference arm: the reference's algorithm on the host cores
# ---------------------------------------------------------------------------------------------

_W = {}


def _worker_init(arrs):
    from flexaidds_gb300.system import Descriptor
    from oracle import port
    d = Descriptor.from_arrays(arrs)
    _W["d"] = d
    _W["o"] = port.Oracle(d)


def _worker_status(genes):
    d = _W["d"]
    return _W["o"].eval_ic(d.genes_to_ic(genes))["cf"]["status"]


def _worker_eval(ic):
    return _W["o"].eval_ic(ic)["cf"]["evalue"]


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import port
    port.build()
    d = make_system()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_worker_init, initargs=(d.to_arrays(),)) as pool:
        def status_of(g):
            parts = np.array_split(g, cores * 4)
            return np.concatenate(pool.map(_worker_status, parts))
        pops = scored_populations(d, 1, status_of)
        ic = d.genes_to_ic(pops[0])
        parts = np.array_split(ic, cores * 4)
        for _ in range(args.warmup):
            pool.map(_worker_eval, parts)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            pool.map(_worker_eval, parts)
        dt = time.perf_counter() - t0
    pop = WORKLOAD["population"]
    value = pop * args.steps / dt
    out = {
        "metric": METRIC, "value": value, "unit": "poses/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Poisson-disc receptor, seeded tree ligand, N(0,1) matrix)",
        "config": {"workload": WORKLOAD_NAME, "population": pop, "precision": "reference",
                   "parallelism": f"{cores} host processes"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "poses/s", "cores": cores, "kind": "port",
                         "sample": f"one population of {pop} per step on {cores} processes of "
                                   f"{cpu_model()}; the C restatement of the reference's "
                                   "ic2cf/Vcontacts/vcfunction (the reference's own sources do "
                                   "not travel to this host)"},
        "e2e": {"value": value, "unit": "poses/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["reference", "fast"], default="reference")
    ap.add_argument("--served", type=int, default=1,
                    help="also serve Poisson streams of docking jobs and report latency percentiles")
    ap.add_argument("--batched", type=int, default=1,
                    help="also time the batched many-ligand workload against one launch per job")
    ap.add_argument("--cluster", type=int, default=1,
                    help="also time the clustering of a 1e6-chromosome ensemble")
    ap.add_argument("--cluster-only", type=int, default=0, metavar="CENTRES",
                    help="time only the clustering, of CENTRES x 500 chromosomes (a small case "
                         "for a profiler: few launches before the clustering kernels)")
    args = ap.parse_args()
    if args.cluster_only:
        from flexaidds_gb300 import evaluator
        d = make_system()
        ev = evaluator.GPUEvaluator(d, max_poses=64)
        print(json.dumps({"cluster": run_cluster(ev, d, centres=args.cluster_only)}), flush=True)
        ev.close()
        return
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
