"""Serving docking jobs on one GPU with continuous batching.

Jobs (a ligand on a cached receptor, a population size, a number of generations, a seed) arrive
over time. Arrived jobs are admitted between generations, first come first served, while job
slots and the device-memory budget allow; every running job advances one generation per engine
step (one CUDA graph of breeding, a batched evaluation of all running jobs' children and
selection, `fxe_ga_step`), and a job leaves the engine as soon as its last generation is done,
freeing its slot and memory for the next arrivals. A job's result (best pose, best energy, the
FP64 thermodynamics of everything it evaluated) depends only on the job, not on what else ran.

Receptors are cached: the first job on a receptor generates its cleft grid and the grid's
internal coordinates on the device (`fxe_cleft_grid`) and creates a context holding the receptor,
its cell list (built on the device) and the grid; every later job on it shares them
(`fxe_context_create_shared`). A job's own preparation (the ligand's build tree, gene limits and
descriptor) happens when it is admitted, so it counts in the job's latency.

`DockingServer(max_jobs=1)` is the plain path served: one job at a time, one population per
launch, the others waiting in arrival order.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import evaluator, prepare
from .evaluator import GAEngine, GPUEvaluator
from .system import Descriptor, SystemInputs


@dataclass
class JobRequest:
    arrival: float          # seconds after the start of the stream
    receptor: str           # key of the receptor in the server's cache
    inputs: SystemInputs    # the job's system (receptor, ligand, matrix), prepared on admission
    population: int = 500
    generations: int = 100
    seed: int = 0
    cross_rate: float = 0.8     # the reference's defaults (LIB/config_parser.cpp:128-129)
    mut_rate: float = 0.03


@dataclass
class JobResult:
    index: int
    arrival: float
    admitted: float
    finished: float
    best_energy: float
    best_genes: np.ndarray
    thermo: dict = field(default_factory=dict)

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def context_bytes(desc: Descriptor, max_poses: int) -> int:
    """Device bytes of a context's per-pose workspace (fxe_context_create's allocations)."""
    P, n, ng = int(max_poses), desc.n_lig, max(1, desc.n_genes)
    per_atom = 96 * (4 + 4 + 8 + 1) + 16 + 4 + 4 + 4 + 8
    return P * (ng * (8 + 4 + 8) + n * per_atom + 16 + 16 + 104) + 4096


class DockingServer:
    """Continuous batching of GA docking jobs behind a receptor cache and a memory budget."""

    def __init__(self, max_jobs: int = 256, hbm_budget: float = 150e9, precision: int = 0,
                 temperature: float = 300.0):
        self.engine = GAEngine(max_jobs, precision)
        self.max_jobs = int(max_jobs)
        self.budget = float(hbm_budget)
        self.precision = int(precision)
        self.temperature = float(temperature)
        self.receptors: dict[str, tuple] = {}   # key -> (receptor setup, context holding the receptor)

    def _receptor(self, key: str, inp: SystemInputs):
        """The cached receptor: its frame and cleft grid ICs (grid on the device) and a context
        whose device arrays later jobs share."""
        if key not in self.receptors:
            rec = inp.receptor
            frame = prepare.calc_center(rec.xyz)
            xyz, ic = evaluator.cleft_grid(rec.cleft_center, [rec.cleft_radius], 0.375, frame[0])
            setup = (frame, ic)
            inp = SystemInputs(receptor=rec, ligand=inp.ligand, grid_xyz=xyz, emat=inp.emat)
            base = GPUEvaluator(prepare.prepare(inp, setup), max_poses=2, precision=self.precision)
            self.receptors[key] = (setup, xyz, base)
        return self.receptors[key]

    def _prepare(self, r: JobRequest) -> tuple:
        setup, xyz, base = self._receptor(r.receptor, r.inputs)
        inp = r.inputs
        desc = prepare.prepare(SystemInputs(receptor=inp.receptor, ligand=inp.ligand, grid_xyz=xyz, emat=inp.emat,
                                            permeability=inp.permeability, dee_clash=inp.dee_clash,
                                            intramolecular=inp.intramolecular, solventterm=inp.solventterm),
                               setup)
        return desc, base

    def run(self, requests: list[JobRequest]) -> list[JobResult]:
        order = sorted(range(len(requests)), key=lambda i: requests[i].arrival)
        pending = list(order)
        running = {}            # slot -> (index, evaluator, admitted, bytes, last step)
        results: list[JobResult] = []
        used = 0.0
        step = 0
        t0 = time.perf_counter()
        while pending or running:
            now = time.perf_counter() - t0
            while pending and requests[pending[0]].arrival <= now and len(running) < self.max_jobs:
                i = pending[0]
                r = requests[i]
                desc, base = self._prepare(r)
                job_bytes = context_bytes(desc, r.population)
                if used + job_bytes > self.budget and running:
                    break
                ev = GPUEvaluator(desc, max_poses=r.population, precision=self.precision,
                                  share_receptor_with=base)
                job = self.engine.job(ev, r.population, r.generations, r.seed, r.cross_rate, r.mut_rate)
                job_bytes += self.engine.job_bytes(job)
                slot = self.engine.admit(job, ev)
                running[slot] = (i, ev, time.perf_counter() - t0, job_bytes, step + r.generations)
                used += job_bytes
                pending.pop(0)
            if not running:
                time.sleep(max(0.0, requests[pending[0]].arrival - (time.perf_counter() - t0)))
                continue
            self.engine.step()
            step += 1
            # the host knows when each job's last generation was queued: wait only then
            if any(last <= step for (_, _, _, _, last) in running.values()):
                for slot in self.engine.finished():
                    i, ev, admitted, job_bytes, _ = running.pop(slot)
                    g, e, th = self.engine.collect(slot, self.temperature)
                    results.append(JobResult(i, requests[i].arrival, admitted, time.perf_counter() - t0, e, g, th))
                    ev.close()
                    used -= job_bytes
        return results

    def close(self):
        self.engine.close()
        for _, _, ev in self.receptors.values():
            ev.close()


def latency_summary(results: list[JobResult]) -> dict:
    lat = np.asarray([r.latency for r in results])
    span = max(r.finished for r in results) - min(r.arrival for r in results)
    return {"jobs": len(results), "jobs_per_s": len(results) / span if span > 0 else None,
            "p50_s": float(np.percentile(lat, 50)), "p95_s": float(np.percentile(lat, 95)),
            "p99_s": float(np.percentile(lat, 99)), "makespan_s": span}


def poisson_arrivals(n: int, rate: float, seed: int) -> np.ndarray:
    """Arrival times (s) of a Poisson stream of n jobs at `rate` jobs/s."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


__all__ = ["DockingServer", "JobRequest", "JobResult", "latency_summary", "poisson_arrivals",
           "context_bytes", "evaluator"]
