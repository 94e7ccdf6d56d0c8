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
# FP64 work per energy of the reduction: the log-weight, the running maximum and its rescaling, one
# exp (counted as 10), the three running sums
STATMECH_FLOP = 20

# DRAM bytes per launch of the dominant kernel from ncu (dram__bytes_read.sum +
# dram__bytes_write.sum), keyed by precision; from profiles/pose_kernel_plain_scale.md.
POSE_KERNEL_DRAM_BYTES = {"reference": 106_995_968, "fast": 99_187_200}

# nominal non-tensor arithmetic peaks of GB300 (152 SMs at 2,070 MHz): FP32 152 x 128 lanes x 2
# flops per FMA; FP64 1.25 TFLOP/s. There is no measured figure for either.
NOMINAL_PEAK_TFLOPS = {"fast": 152 * 128 * 2 * 2.07e9 / 1e12, "reference": 1.25}


def bench_config(prec: str) -> dict:
    """The workload as both arms name it (the same dict in both JSON lines)."""
    w = WORKLOAD
    return {"workload": WORKLOAD_NAME, "population": w["population"], "precision": prec,
            "side_chains": f"{w['side_chains']} residues x {w['rotamers']} rotamers"}


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
    # receptors of the many-receptor legs, generated on the host cores before anything is timed
    pool = futs4 = futs5 = None
    if args.batched or args.served:
        specs4 = receptor_specs(BATCH4["receptors"], BATCH4["seed"], side_chains=True) if args.batched else []
        specs5 = receptor_specs(SERVE["receptors"], SERVE["seed"], side_chains=False) if args.served else []
        pool, futs = start_receptor_pool(specs4 + specs5)
        futs4, futs5 = futs[:len(specs4)], futs[len(specs4):]
        rec4 = [f.result() for f in futs4]
        rec5 = [f.result() for f in futs5]
        pool.shutdown()
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

    # the polyhedron launch's occupancy cap for this size class, tuned on the first population
    sweep = ev.autotune_sweep(dgen[0].data_ptr(), pop, reps=2)
    tuned_cap = min(sweep, key=lambda c: (sweep[c], c))
    tuned_ms = sweep[tuned_cap]
    # and the contact scan's form (cell entries read in place, or staged in shared memory)
    cells = ev.autotune_contacts(dgen[0].data_ptr(), pop, reps=3)

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
    e2e_steps = []
    barrier()
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        rc = lib.fxe_eval_genes(ev.handle, pop, C.cast(hgen[k % N_POPULATIONS].data_ptr(), capi._i),
                                C.c_void_p(hout.data_ptr()))
        e2e_steps.append(time.perf_counter() - t)
        e2e_s += e2e_steps[-1]
        if rc != 0:
            raise RuntimeError(lib.fxe_last_error().decode())
    barrier()
    e2e_s = max_over_ranks(e2e_s)
    res = np.frombuffer(hout.numpy().tobytes(), capi.CF_DTYPE)
    assert np.all(res["status"] != capi.POSE_CAPACITY)

    # --- statmech over a run's ensemble (1e6 poses, FP64) -------------------------------------
    # fxe_thermo_compute_device_fixed: the reduction and its merge on the device, the record
    # written to device memory (kernel time, no host round trip); fxe_thermo_compute_device: the
    # same with the merge on the host (the call waits for it)
    from flexaidds_gb300.capi import Thermo
    energies = torch.from_numpy(np.random.default_rng(1).normal(-30.0, 5.0, STATMECH_N)).cuda()
    th = Thermo()
    d_th = torch.zeros(C.sizeof(Thermo), dtype=torch.uint8, device="cuda")

    lib.fxe_thermo_compute_device_fixed.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_void_p,
                                                    C.c_void_p]

    def thermo_fixed():
        rc = lib.fxe_thermo_compute_device_fixed(C.c_void_p(energies.data_ptr()), None, STATMECH_N, 300.0,
                                                 C.c_void_p(d_th.data_ptr()), C.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.fxe_last_error().decode())

    def thermo_host_merge():
        lib.fxe_thermo_compute_device(C.c_void_p(energies.data_ptr()), None, STATMECH_N, 300.0,
                                      C.byref(th), C.c_void_p(stream.cuda_stream))

    sm = {}
    for nm, fn in (("device_merge", thermo_fixed), ("host_merge", thermo_host_merge)):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        best = None
        for _ in range(10):
            flush.zero_()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            t = a.elapsed_time(b)
            best = t if best is None else min(best, t)
        sm[nm] = best
    sm_best = sm["device_merge"]

    clustered = run_cluster(ev, d) if args.cluster else None
    batched = batched4 = batched_fp32 = None
    if args.batched:
        batched = run_batched(args, prec, flush, stream, BATCH_NAME, c3_jobs(), BATCH["evolve"])
        batched4 = run_batched(args, prec, flush, stream, BATCH4_NAME, c4_jobs(rec4), BATCH4["evolve"])
        # the 256-ligand workload names FP32 geometry: the same comparison in fast precision
        batched_fp32 = run_batched(args, "fast", flush, stream, BATCH_NAME, c3_jobs(), BATCH["evolve"])
    served = run_served(prec, rec5) if args.served else None
    ga_runs = {k: run_ga(prec, k, d if k == "c2" else None) for k in ("c1", "c2")} if args.ga else None

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
    sm_tflops = STATMECH_FLOP * STATMECH_N / (sm_best / 1e3) / 1e12
    try:
        cpu = cpu_baseline_port(d, pops)
    except Exception as e:   # the oracle library could not be built or loaded
        cpu = {"value": None, "unit": "poses/s", "cores": 1, "kind": "port", "sample": f"unavailable: {e}"}

    out = {
        "metric": METRIC, "value": value, "unit": "poses/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == "reference" else "f32",
        "data": "synthetic (seeded Poisson-disc receptor, seeded tree ligand, N(0,1) matrix)",
        "config": bench_config(prec),
        "l2": f"flushed between timed steps ({FLUSH_BYTES >> 20} MB write)",
        "parallelism": f"replicas x{world}",
        "e2e": {"value": world * pop * args.steps / e2e_s, "unit": "poses/s",
                "step_ms": {"median": 1e3 * float(np.median(e2e_steps)), "min": 1e3 * min(e2e_steps),
                            "max": 1e3 * max(e2e_steps)},
                "h2d_bytes_per_step": pop * d.n_genes * 4, "d2h_bytes_per_step": pop * capi.CF_DTYPE.itemsize},
        "gpu_launches": launches,
        "autotune": {"pose_blocks_per_sm": tuned_cap, "launch_ms": tuned_ms,
                     "sweep_ms": {str(c): round(t, 3) for c, t in sorted(sweep.items())},
                     "contacts_ms": {"in_place": round(cells["in_place_ms"], 4),
                                     "staged": round(cells["staged_ms"], 4)},
                     "contacts_staged": cells["staged"]},
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
                     "ms_host_merge": sm["host_merge"],
                     "roofline": {"bound": "fp64", "achieved": sm_tflops, "peak": NOMINAL_PEAK_TFLOPS["reference"],
                                  "unit": "TFLOP/s", "frac": sm_tflops / NOMINAL_PEAK_TFLOPS["reference"],
                                  "flop_per_energy": STATMECH_FLOP, "peak_source": "nominal FP64",
                                  "hbm_gbs": sm_gbs, "hbm_frac": (sm_gbs / hbm) if hbm else None,
                                  "traffic": None}},
        "batched": batched,
        "batched_c4": batched4,
        "batched_fp32": batched_fp32,
        "served": served,
        "ga": ga_runs,
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
# receptors of the many-receptor workloads: generated in worker processes (spawned, no CUDA)
# ---------------------------------------------------------------------------------------------

def receptor_specs(n, seed, side_chains):
    """n seeded receptor shapes of 1,500-8,000 atoms and 6-14 A clefts; with side_chains, 0-4
    flexible side chains of 4-12 rotamers each."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        out.append(dict(n_rec=int(rng.integers(1500, 8001)), cleft=float(rng.uniform(6.0, 14.0)),
                        side_chains=int(rng.integers(0, 5)) if side_chains else 0,
                        rotamers=int(rng.integers(4, 13)), seed=int(seed * 100 + k)))
    return out


def _gen_receptor(spec):
    return system.make_inputs(spec["n_rec"], spec["cleft"], 12, 3, seed=spec["seed"],
                              side_chains=spec["side_chains"], rotamers=spec["rotamers"])


def start_receptor_pool(specs):
    """Futures of the receptors' inputs, generated by a pool of spawned processes."""
    import concurrent.futures as cf
    import multiprocessing as mp
    ex = cf.ProcessPoolExecutor(max_workers=max(1, min(len(specs), os.cpu_count() or 1)),
                                mp_context=mp.get_context("spawn"))
    return ex, [ex.submit(_gen_receptor, s) for s in specs]


# ---------------------------------------------------------------------------------------------
# batched: many ligands (on one receptor, or on many), one launch per generation
# ---------------------------------------------------------------------------------------------

BATCH = dict(n_rec=4000, cleft=10.0, seed=31, edge=51.92391670510951, jobs=256, atoms=(10, 70),
             torsions=(0, 15), population=(200, 2000), evolve=5)
BATCH_NAME = ("batched C3: 4000-atom receptor, 10 A cleft (79501 grid points), 256 seeded ligands of "
              "U[10,70] heavy atoms and U[0,15] torsions, populations U[200,2000] after 5 GA "
              "generations on the device; one generation's evaluation of every job per step")
BATCH4 = dict(receptors=16, ligands=32, population=500, atoms=(10, 70), torsions=(0, 15), seed=44, evolve=5)
BATCH4_NAME = ("batched C4: 16 seeded receptors of 1500-8000 atoms (6-14 A clefts, 0-4 flexible side "
               "chains of 4-12 rotamers), 32 ligands each (U[10,70] heavy atoms, U[0,15] torsions), 512 "
               "jobs of population 500 after 5 GA generations on the device; one generation's "
               "evaluation of every job per step")


def c3_jobs():
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
        out.append(("c3", SystemInputs(receptor=base.receptor, ligand=lig, grid_xyz=base.grid_xyz,
                                       emat=base.emat), pop))
    return out


def c4_jobs(receptors):
    from flexaidds_gb300.system import SystemInputs
    b = BATCH4
    rng = np.random.default_rng(b["seed"])
    out = []
    for r, base in enumerate(receptors):
        for k in range(b["ligands"]):
            n = int(rng.integers(b["atoms"][0], b["atoms"][1] + 1))
            t = int(rng.integers(b["torsions"][0], b["torsions"][1] + 1))
            lig = synth.random_ligand(n, t, seed=b["seed"] * 100000 + r * 1000 + k)
            out.append((f"r{r}", SystemInputs(receptor=base.receptor, ligand=lig, grid_xyz=base.grid_xyz,
                                              emat=base.emat), b["population"]))
    return out


def evolved_populations(jobs, prec, generations, seed):
    """Contexts of the jobs (one receptor copy per receptor key) and each job's population after
    `generations` GA generations on the device (the reference's defaults)."""
    from flexaidds_gb300 import evaluator
    p = 0 if prec == "reference" else 1
    bases, evs = {}, []
    for key, inp, pop in jobs:
        d = prepare.prepare(inp)
        if key not in bases:
            bases[key] = evaluator.GPUEvaluator(d, max_poses=pop, precision=p)
            evs.append(bases[key])
        else:
            evs.append(evaluator.GPUEvaluator(d, max_poses=pop, precision=p, share_receptor_with=bases[key]))
    eng = evaluator.GAEngine(max_jobs=len(jobs), precision=p)
    slots = [eng.admit(eng.job(ev, pop, generations + 1, seed * 7919 + k), ev)
             for k, (ev, (_, _, pop)) in enumerate(zip(evs, jobs))]
    for _ in range(generations):
        eng.step()
    genes = [eng.read_population(sl, pop)[0] for sl, (_, _, pop) in zip(slots, jobs)]
    eng.close()
    return evs, genes


def run_batched(args, prec, flush, stream, name, jobs, generations):
    """Poses/s of one generation's evaluation of all jobs (their evolved populations): one launch
    sequence per job (the plain path) and one batched launch for all of them, same chromosomes,
    device-resident, L2 flushed."""
    import torch
    from flexaidds_gb300 import evaluator
    t_setup = time.perf_counter()
    evs, genes = evolved_populations(jobs, prec, generations, seed=len(jobs))
    setup_s = time.perf_counter() - t_setup
    pops = [g.shape[0] for g in genes]
    dg = [torch.from_numpy(np.ascontiguousarray(g)).cuda() for g in genes]
    do = [torch.empty(pop * capi.CF_DTYPE.itemsize, dtype=torch.uint8, device="cuda") for pop in pops]
    total = sum(pops)
    batch = evaluator.Batch(max_jobs=len(jobs), max_poses=total, max_genes=64)
    table = [(ev, pop, g.data_ptr(), o.data_ptr()) for ev, pop, g, o in zip(evs, pops, dg, do)]

    def plain():
        for ev, pop, g, o in table:
            ev.eval_genes_device(g, pop, o, stream.cuda_stream)

    def batched():
        batch.eval_genes_device(table, stream.cuda_stream)

    res = {}
    steps = max(1, min(args.steps, 3))
    for nm, fn in (("plain", plain), ("batched", batched)):
        with torch.cuda.stream(stream):
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
        res[nm] = {"poses_per_s": total * steps / (ms / 1e3), "ms_per_generation": ms / steps}
    batched_out = [np.frombuffer(o.cpu().numpy().tobytes(), capi.CF_DTYPE) for o in do]
    plain()
    stream.synchronize()
    plain_out = [np.frombuffer(o.cpu().numpy().tobytes(), capi.CF_DTYPE) for o in do]
    same = all(np.array_equal(a, b) for a, b in zip(batched_out, plain_out))
    scored = sum(int((o["status"] == capi.POSE_SCORED).sum()) for o in plain_out)
    for ev in evs:
        ev.close()
    batch.close()
    return {"workload": name, "jobs": len(jobs), "poses_per_generation": total,
            "scored_fraction": scored / total, "precision": prec, "steps": steps,
            "plain": res["plain"], "batched": res["batched"],
            "speedup": res["batched"]["poses_per_s"] / res["plain"]["poses_per_s"],
            "results_identical": same, "setup_s": setup_s}


# ---------------------------------------------------------------------------------------------
# served: Poisson arrivals of docking jobs, continuous batching on the device GA engine
# ---------------------------------------------------------------------------------------------

SERVE = dict(receptors=32, jobs=48, population=500, generations=100, budget=150e9, atoms_median=30,
             atoms=(10, 70), torsions=(0, 15), seed=77, load=(0.5, 0.9, 1.5), plain_jobs=12)
SERVE_NAME = ("served C5 (scaled: 48 jobs per stream where the config has 10,000): receptors from a "
              "cache of 32 seeded receptors of 1500-8000 atoms (6-14 A clefts), ligands lognormal "
              "median 30 heavy atoms (10-70) with U[0,15] torsions, population 500 for 100 generations, "
              "the reference's GA defaults (PSHARE fitness, BOOM, duplicates rejected), 150 GB "
              "admission budget; the receptor's grid and each job's descriptor prepared on admission, "
              "inside the job's latency. Capacity first (all jobs at t = 0), then Poisson streams at "
              "0.5, 0.9 and 1.5 times it, and the plain path (one job at a time, the first 12 jobs) at 0.5 "
              "times it")


def run_served(prec, receptors):
    from flexaidds_gb300 import serve
    from flexaidds_gb300.system import SystemInputs
    s = SERVE
    rng = np.random.default_rng(s["seed"])
    reqs = []
    for k in range(s["jobs"]):
        r = int(rng.integers(len(receptors)))
        base = receptors[r]
        n = int(np.clip(round(rng.lognormal(np.log(s["atoms_median"]), 0.4)), *s["atoms"]))
        t = int(rng.integers(s["torsions"][0], s["torsions"][1] + 1))
        lig = synth.random_ligand(n, t, seed=s["seed"] * 1000 + k)
        inp = SystemInputs(receptor=base.receptor, ligand=lig, grid_xyz=base.grid_xyz, emat=base.emat)
        reqs.append(serve.JobRequest(0.0, f"r{r}", inp, s["population"], s["generations"], seed=s["seed"] * 7919 + k))
    p = 0 if prec == "reference" else 1

    def serve_once(arrivals, max_jobs):
        for q, t in zip(reqs, arrivals):
            q.arrival = float(t)
        srv = serve.DockingServer(max_jobs=max_jobs, hbm_budget=s["budget"], precision=p)
        res = srv.run(reqs)
        launches, graphs = srv.engine.take_launches()
        srv.close()
        summ = serve.latency_summary(res)
        poses = len(res) * s["population"] * (s["generations"] + 1)
        summ.update({"poses_per_s": poses / summ["makespan_s"], "graph_launches": graphs,
                     "kernel_launches": launches})
        return summ

    out = {"workload": SERVE_NAME, "precision": prec, "jobs_per_stream": s["jobs"]}
    cap = serve_once(np.zeros(len(reqs)), 256)
    capacity = cap["jobs_per_s"]
    out["capacity"] = dict(cap, arrival_rate=None)
    out["rates"] = []
    for f in s["load"]:
        rate = capacity * f
        summ = serve_once(serve.poisson_arrivals(len(reqs), rate, seed=int(1000 * f)), 256)
        summ.update({"arrival_rate": rate, "load": f})
        out["rates"].append(summ)
    rate = capacity * s["load"][0]
    del reqs[s["plain_jobs"]:]
    plain = serve_once(serve.poisson_arrivals(len(reqs), rate, seed=int(1000 * s["load"][0])), 1)
    plain.update({"arrival_rate": rate, "load": s["load"][0], "jobs": len(reqs)})
    out["plain"] = plain
    return out


# ---------------------------------------------------------------------------------------------
# whole GA runs: C1 (500 x 100 generations) and C2 (2000 x 500 generations, 1e6 poses) on the
# device GA engine, ensemble and thermodynamics included
# ---------------------------------------------------------------------------------------------

GA_RUNS = {
    "c1": dict(n_rec=2000, cleft=8.0, n_lig=24, n_tor=6, seed=11, edge=None, side_chains=0, rotamers=8,
               population=500, generations=100,
               name="C1: 2000-atom receptor, 8 A cleft, 24-atom ligand, 6 torsions, population 500 for 100 generations"),
    "c2": dict(n_rec=6000, cleft=12.0, n_lig=48, n_tor=12, seed=7, edge=WORKLOAD["edge"], side_chains=3, rotamers=8,
               population=2000, generations=500,
               name="C2: the plain-scale system (6000 atoms, 3 side chains of 8 rotamers, 48-atom ligand, 12 "
                    "torsions), population 2000 for 500 generations (1e6 poses)"),
}


def run_ga(prec, key, d=None):
    """One docking job's whole GA on the device: poses/s over the run, the ensemble's size and the
    FP64 thermodynamics of it at 300 K."""
    import torch
    from flexaidds_gb300 import evaluator
    g = GA_RUNS[key]
    if d is None:
        d = prepare.prepare(system.make_inputs(g["n_rec"], g["cleft"], g["n_lig"], g["n_tor"], seed=g["seed"],
                                               edge=g["edge"], side_chains=g["side_chains"], rotamers=g["rotamers"]))
    p = 0 if prec == "reference" else 1
    ev = evaluator.GPUEvaluator(d, max_poses=g["population"], precision=p)
    eng = evaluator.GAEngine(max_jobs=1, precision=p)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    slot = eng.admit(eng.job(ev, g["population"], g["generations"], seed=2024), ev)
    for _ in range(g["generations"]):
        eng.step()
    assert eng.finished() == [slot]
    t1 = time.perf_counter()
    best_g, best_e, th = eng.collect(slot, 300.0)
    t2 = time.perf_counter()
    eng.close()
    ev.close()
    poses = g["population"] * (g["generations"] + 1)
    return {"workload": g["name"], "precision": prec, "poses": poses, "seconds": t1 - t0,
            "poses_per_s": poses / (t1 - t0), "collect_s": t2 - t1, "best_energy": best_e,
            "n_ensemble": th["n_ensemble"], "free_energy": th["free_energy"],
            "mean_energy": th["mean_energy"], "minus_T_dS": -300.0 * th["entropy"],
            "heat_capacity": th["heat_capacity"]}


def run_thermo_only(n, reps=20):
    """fxe_thermo_compute_device_fixed over n seeded energies (N(-30, 5) kcal/mol) at 300 K: the
    best CUDA-event time of reps calls after three warm-up calls, and the record it wrote."""
    import ctypes as C
    import torch
    from flexaidds_gb300 import evaluator
    from flexaidds_gb300.capi import Thermo
    lib = evaluator.load_library()
    lib.fxe_thermo_compute_device_fixed.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_void_p,
                                                    C.c_void_p]
    e = torch.from_numpy(np.random.default_rng(1).normal(-30.0, 5.0, n)).cuda()
    d_th = torch.zeros(C.sizeof(Thermo), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def call():
        rc = lib.fxe_thermo_compute_device_fixed(C.c_void_p(e.data_ptr()), None, n, 300.0,
                                                 C.c_void_p(d_th.data_ptr()), C.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(lib.fxe_last_error().decode())

    for _ in range(3):
        call()
    torch.cuda.synchronize()
    best = None
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        call()
        b.record(stream)
        b.synchronize()
        t = a.elapsed_time(b)
        best = t if best is None else min(best, t)
    th = Thermo.from_buffer_copy(d_th.cpu().numpy().tobytes())
    return {"n": n, "best_ms": best, "free_energy": th.free_energy, "mean_energy": th.mean_energy}


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
        "config": bench_config(args.precision),
        "parallelism": f"{cores} host processes",
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
    ap.add_argument("--ga", type=int, default=1,
                    help="also run whole GA jobs: C1 (500 x 100 generations) and C2 (2000 x 500)")
    ap.add_argument("--cluster-only", type=int, default=0, metavar="CENTRES",
                    help="time only the clustering, of CENTRES x 500 chromosomes (a small case "
                         "for a profiler: few launches before the clustering kernels)")
    ap.add_argument("--ga-only", default="", metavar="KEY:GENERATIONS",
                    help="run only one whole GA job, e.g. c2:40 (a small case for a profiler)")
    ap.add_argument("--thermo-only", type=int, default=0, metavar="N",
                    help="time only the device-merged thermodynamics of N energies (a small case "
                         "for a profiler)")
    args = ap.parse_args()
    if args.ga_only:
        key, _, gens = args.ga_only.partition(":")
        if gens:
            GA_RUNS[key]["generations"] = int(gens)
            GA_RUNS[key]["name"] += f"; this run: {int(gens)} generations"
        print(json.dumps({"ga": run_ga(args.precision, key)}), flush=True)
        return
    if args.thermo_only:
        print(json.dumps({"thermo": run_thermo_only(args.thermo_only)}), flush=True)
        return
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
