"""Host-side interface of the GB300 evaluation backend (ctypes over libfxe.so).

Mirrors the reference's evaluation entry points for this path:
  * ``GPUEvaluator``   — the CUDA backend of calculate_fitness (cuda_eval_init / cuda_eval_batch /
                         cuda_eval_shutdown, LIB/cuda_eval.cuh:46-75), scoring whole batches and
                         returning the full cfstr per pose instead of the surrogate's com/wal/sas;
  * ``ic2cf``          — single-pose scoring with the signature's meaning (LIB/ic2cf.cpp:18);
  * ``StatMechEngine`` — add_sample / compute / boltzmann_weights / delta_G / helmholtz
                         (LIB/statmech.h:67-135) with the reduction on the device in FP64.

There is no CPU fallback: without the built library or a CUDA device these raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .capi import CF_DTYPE, STATUS_NAMES, Packed, Thermo, _d, _f, _i, ptr
from .system import Descriptor

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libfxe.so")
_lib = None


class FxeError(RuntimeError):
    pass


def load_library():
    """Loads flexaidds_gb300/libfxe.so (built by flexaidds_gb300/build.py)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FxeError(f"CUDA backend not built: {LIB_PATH} is missing (run flexaidds_gb300/build.py)")
        lib = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        lib.fxe_context_create.argtypes = [vp, vp, vp, vp, C.c_int32, C.POINTER(vp)]
        lib.fxe_eval_genes.argtypes = [vp, C.c_int32, _i, vp]
        lib.fxe_eval_ic.argtypes = [vp, C.c_int32, _d, vp]
        lib.fxe_eval_genes_device.argtypes = [vp, C.c_int32, vp, vp, vp]
        lib.fxe_last_contacts.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, _i, _f, _i]
        lib.fxe_last_stats.argtypes = [vp, _i]
        lib.fxe_last_ligand_xyz.argtypes = [vp, C.c_int32, _f]
        lib.fxe_thermo_compute.argtypes = [_d, _i, C.c_int64, C.c_double, vp]
        lib.fxe_thermo_compute_device.argtypes = [vp, vp, C.c_int64, C.c_double, vp, vp]
        lib.fxe_thermo_weights.argtypes = [_d, _i, C.c_int64, C.c_double, _d]
        lib.fxe_context_set_precision.argtypes = [vp, C.c_int32]
        lib.fxe_context_set_face_order.argtypes = [vp, C.c_int32]
        lib.fxe_context_set_cell_staging.argtypes = [vp, C.c_int32]
        lib.fxe_context_enable_timing.argtypes = [vp, C.c_int32]
        lib.fxe_context_take_timing.argtypes = [vp, _d, C.POINTER(C.c_int64)]
        lib.fxe_context_create_shared.argtypes = [vp, vp, vp, vp, C.c_int32, C.POINTER(vp)]
        lib.fxe_batch_create.argtypes = [C.c_int32, C.c_int64, C.c_int32, C.POINTER(vp)]
        lib.fxe_batch_eval_genes.argtypes = [vp, vp, C.c_int32]
        lib.fxe_batch_eval_genes_device.argtypes = [vp, vp, C.c_int32, vp]
        lib.fxe_batch_take_launches.argtypes = [vp, C.POINTER(C.c_int64)]
        lib.fxe_batch_destroy.argtypes = [vp]
        lib.fxe_batch_destroy.restype = None
        lib.fxe_ga_create.argtypes = [C.c_int32, C.c_int32, C.POINTER(vp)]
        lib.fxe_ga_job_bytes.argtypes = [vp, C.POINTER(C.c_int64)]
        lib.fxe_ga_admit.argtypes = [vp, vp, C.POINTER(C.c_int32)]
        lib.fxe_ga_step.argtypes = [vp]
        lib.fxe_ga_finished.argtypes = [vp, _i, C.c_int32, C.POINTER(C.c_int32)]
        lib.fxe_ga_collect.argtypes = [vp, C.c_int32, C.c_double, _i, C.POINTER(C.c_double), vp,
                                       C.POINTER(C.c_int64)]
        lib.fxe_ga_population.argtypes = [vp, C.c_int32, _i, _d]
        lib.fxe_ga_ensemble.argtypes = [vp, C.c_int32, C.c_int64, _d, _d, C.POINTER(C.c_int64)]
        lib.fxe_ga_take_launches.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        lib.fxe_ga_duplicates.argtypes = [vp, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        lib.fxe_ga_destroy.argtypes = [vp]
        lib.fxe_ga_destroy.restype = None
        lib.fxe_cluster.argtypes = [vp, C.c_int64, _d, _d, C.c_int32, C.c_float, C.c_int32, _i, _i, _d, _d,
                                    _i, _f, _f, _i]
        lib.fxe_last_cluster_time.argtypes = [vp, _d]
        lib.fxe_decode_genes.argtypes = [vp, C.c_int64, _i, C.c_int32, _d]
        lib.fxe_ga_breed_draws.argtypes = [C.c_int32, C.c_int32, _i, _d, _i, _f, C.c_double, C.c_double,
                                           C.c_int32, C.c_int32, _d, C.c_int32, _d, _i, _i, _d]
        lib.fxe_ga_niche_counts.argtypes = [C.c_int32, C.c_int32, _d, C.c_double, C.c_double, _d]
        lib.fxe_ensemble_dedup.argtypes = [C.c_int64, C.c_int32, _d, _d, C.POINTER(C.c_int64), _d,
                                           C.POINTER(C.c_int64)]
        lib.fxe_cleft_grid.argtypes = [C.c_int32, _f, _f, C.c_float, _f, C.c_int64, _f, _f, C.POINTER(C.c_int64)]
        lib.fxe_context_autotune.argtypes = [vp, C.c_int32, vp, C.c_int32, C.POINTER(C.c_int32),
                                             C.POINTER(C.c_double)]
        lib.fxe_context_autotune_sweep.argtypes = [vp, C.c_int32, vp, C.c_int32, _i, _d, C.c_int32,
                                                   C.POINTER(C.c_int32)]
        lib.fxe_autotune_lookup.argtypes = [C.c_int32, C.c_int32, C.c_int64, C.POINTER(C.c_int32)]
        lib.fxe_context_autotune_contacts.argtypes = [vp, C.c_int32, vp, C.c_int32, _d, C.POINTER(C.c_int32)]
        lib.fxe_context_destroy.argtypes = [vp]
        lib.fxe_context_destroy.restype = None
        lib.fxe_last_error.restype = C.c_char_p
        _lib = lib
    return _lib


def _check(rc: int):
    if rc != 0:
        msg = load_library().fxe_last_error().decode()
        raise FxeError(f"{STATUS_NAMES.get(rc, rc)}: {msg}")


class GPUEvaluator:
    """Evaluation context for one receptor, ligand and energy matrix."""

    REFERENCE, FAST = 0, 1
    # how a face whose first point has no neighbour on its second plane is ordered
    # (fxe_context_set_face_order): as the reference does it, or from the point's other plane
    FACE_ORDER_REFERENCE, FACE_ORDER_GEOMETRIC = 0, 1
    # how the contact-candidate scan reads the cell list (fxe_context_set_cell_staging): the
    # autotuner's choice, in place, or staged in shared memory by bulk copies
    CELLS_AUTO, CELLS_IN_PLACE, CELLS_STAGED = 0, 1, 2

    def __init__(self, desc: Descriptor, max_poses: int = 2048, precision: int = 0,
                 share_receptor_with: "GPUEvaluator | None" = None, face_order: int = 0,
                 cell_staging: int = 0):
        """share_receptor_with: an evaluator on the same receptor whose device copy of the
        receptor, cell list and cleft grid this one reuses (fxe_context_create_shared)."""
        self.lib = load_library()
        self.desc = desc
        self._packed = Packed(desc)
        self.max_poses = int(max_poses)
        h = C.c_void_p()
        pk = self._packed
        if share_receptor_with is not None:
            _check(self.lib.fxe_context_create_shared(share_receptor_with.handle, C.byref(pk.lig),
                                                      C.byref(pk.emat), C.byref(pk.params),
                                                      self.max_poses, C.byref(h)))
        else:
            _check(self.lib.fxe_context_create(C.byref(pk.rec), C.byref(pk.lig), C.byref(pk.emat),
                                               C.byref(pk.params), self.max_poses, C.byref(h)))
        self.handle = h
        _check(self.lib.fxe_context_set_precision(self.handle, int(precision)))
        _check(self.lib.fxe_context_set_face_order(self.handle, int(face_order)))
        _check(self.lib.fxe_context_set_cell_staging(self.handle, int(cell_staging)))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.fxe_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def eval_genes(self, genes: np.ndarray) -> np.ndarray:
        genes = np.ascontiguousarray(genes, np.int32)
        out = np.zeros(genes.shape[0], CF_DTYPE)
        _check(self.lib.fxe_eval_genes(self.handle, genes.shape[0], ptr(genes, _i),
                                       out.ctypes.data_as(C.c_void_p)))
        return out

    def eval_ic(self, ic: np.ndarray) -> np.ndarray:
        ic = np.ascontiguousarray(ic, np.float64)
        out = np.zeros(ic.shape[0], CF_DTYPE)
        _check(self.lib.fxe_eval_ic(self.handle, ic.shape[0], ptr(ic, _d), out.ctypes.data_as(C.c_void_p)))
        return out

    def eval_genes_device(self, d_genes: int, n: int, d_out: int, stream: int = 0):
        """Queues a batch whose genes and records are device pointers (not waited for)."""
        _check(self.lib.fxe_eval_genes_device(self.handle, n, C.c_void_p(d_genes), C.c_void_p(d_out),
                                              C.c_void_p(stream) if stream else None))

    def contacts(self, pose: int, atom: int):
        cap = 512
        part = np.zeros(cap, np.int32)
        area = np.zeros(cap, np.float32)
        n = C.c_int32(0)
        _check(self.lib.fxe_last_contacts(self.handle, pose, atom, cap, ptr(part, _i), ptr(area, _f),
                                          C.byref(n)))
        return part[:n.value].copy(), area[:n.value].copy()

    def enable_timing(self, on: bool = True):
        _check(self.lib.fxe_context_enable_timing(self.handle, 1 if on else 0))

    def take_timing(self):
        """(ms per stage [build, candidates, polyhedra+scoring], kernels launched) since the last call."""
        ms = np.zeros(3, np.float64)
        n = C.c_int64(0)
        _check(self.lib.fxe_context_take_timing(self.handle, ptr(ms, _d), C.byref(n)))
        return ms, int(n.value)

    def ligand_xyz(self, pose: int) -> np.ndarray:
        out = np.zeros((self.desc.n_lig, 3), np.float32)
        _check(self.lib.fxe_last_ligand_xyz(self.handle, pose, ptr(out, _f)))
        return out

    def cluster(self, ic: np.ndarray, app_evalue: np.ndarray, temperature: int = 0, rmsd: float = 2.0,
                max_results: int = 10) -> dict:
        """CF-based clustering of a docking result (cluster, LIB/cluster.cpp:9-182) on the device:
        ic (n, n_genes) decoded ICs within their gene limits, best first (the GA's ensemble),
        app_evalue (n,). temperature (K, integer; 0 = the reference's default), rmsd
        (FA->cluster_rmsd) and max_results (FA->max_results) as the reference's options.
        Returns n_clusters and, per cluster entry in the reference's final order, top (head
        chromosome), freq, tcf, acf; per chromosome member_of (head, -1 = unclustered) and rmsd;
        top_rmsd (entries x entries), the RMSD between entry heads listed in the .cad file."""
        ic = np.ascontiguousarray(ic, np.float64)
        e = np.ascontiguousarray(app_evalue, np.float64)
        if ic.ndim != 2 or ic.shape[1] != self.desc.n_genes or e.shape != (ic.shape[0],):
            raise FxeError("cluster: ic must be (n, n_genes) and app_evalue (n,)")
        n, R = ic.shape[0], int(max_results)
        top, freq = np.zeros(R, np.int32), np.zeros(R, np.int32)
        tcf, acf = np.zeros(R, np.float64), np.zeros(R, np.float64)
        member, rms = np.zeros(n, np.int32), np.zeros(n, np.float32)
        top_rmsd = np.zeros((R, R), np.float32)
        nc = C.c_int32(0)
        _check(self.lib.fxe_cluster(self.handle, n, ptr(ic, _d), ptr(e, _d), int(temperature), float(rmsd), R,
                                    ptr(top, _i), ptr(freq, _i), ptr(tcf, _d), ptr(acf, _d), ptr(member, _i),
                                    ptr(rms, _f), ptr(top_rmsd, _f), C.byref(nc)))
        return {"n_clusters": nc.value, "top": top, "freq": freq, "tcf": tcf, "acf": acf,
                "member_of": member, "rmsd": rms, "top_rmsd": top_rmsd}

    def cluster_time(self) -> float:
        """Device milliseconds of the last cluster call's kernels."""
        ms = np.zeros(1, np.float64)
        _check(self.lib.fxe_last_cluster_time(self.handle, ptr(ms, _d)))
        return float(ms[0])

    def autotune(self, d_genes: int, n: int, reps: int = 2) -> tuple:
        """fxe_context_autotune over n device chromosomes: (blocks per SM chosen, its launch ms)."""
        b, ms = C.c_int32(0), C.c_double(0.0)
        _check(self.lib.fxe_context_autotune(self.handle, int(n), C.c_void_p(d_genes), int(reps), C.byref(b),
                                             C.byref(ms)))
        return int(b.value), float(ms.value)

    def autotune_contacts(self, d_genes: int, n: int, reps: int = 2) -> dict:
        """fxe_context_autotune_contacts: the contact launch's fastest ms with the cell entries read
        in place and staged in shared memory, and whether staging was chosen."""
        ms, st = np.zeros(2, np.float64), C.c_int32(0)
        _check(self.lib.fxe_context_autotune_contacts(self.handle, int(n), C.c_void_p(d_genes), int(reps), ptr(ms, _d),
                                                      C.byref(st)))
        return {"in_place_ms": float(ms[0]), "staged_ms": float(ms[1]), "staged": bool(st.value)}

    def autotune_sweep(self, d_genes: int, n: int, reps: int = 2) -> dict:
        """fxe_context_autotune_sweep: {blocks per SM: fastest launch ms} for every cap timed."""
        caps, ms, k = np.zeros(32, np.int32), np.zeros(32, np.float64), C.c_int32(0)
        _check(self.lib.fxe_context_autotune_sweep(self.handle, int(n), C.c_void_p(d_genes), int(reps), ptr(caps, _i),
                                                   ptr(ms, _d), 32, C.byref(k)))
        return {int(c): float(t) for c, t in zip(caps[:k.value], ms[:k.value])}

    def decode_genes(self, genes: np.ndarray, clamp: bool = False) -> np.ndarray:
        """genetoic of every gene on the device (fxe_decode_genes); clamp as eval_chromosome."""
        genes = np.ascontiguousarray(genes, np.int32).reshape(-1, self.desc.n_genes)
        out = np.empty(genes.shape, np.float64)
        _check(self.lib.fxe_decode_genes(self.handle, genes.shape[0], ptr(genes, _i), int(bool(clamp)), ptr(out, _d)))
        return out

    def stats(self) -> dict:
        o = np.zeros(4, np.int32)
        _check(self.lib.fxe_last_stats(self.handle, ptr(o, _i)))
        return {"hull_failures": int(o[1]), "capacity": int(o[2]), "no_partner_faces": int(o[3]),
                "unreplayed_faces": int(o[0])}


class Job(C.Structure):
    _fields_ = [("ctx", C.c_void_p), ("n", C.c_int32), ("genes", C.c_void_p), ("out", C.c_void_p)]


class Batch:
    """Several evaluators' populations scored in one launch of each kernel (fxe_batch_*)."""

    def __init__(self, max_jobs: int, max_poses: int, max_genes: int = 64):
        self.lib = load_library()
        h = C.c_void_p()
        _check(self.lib.fxe_batch_create(int(max_jobs), int(max_poses), int(max_genes), C.byref(h)))
        self.handle = h

    def eval_genes(self, jobs) -> list:
        """jobs: [(GPUEvaluator, int32 genes (n, n_genes)), ...] -> list of record arrays."""
        arr = (Job * max(1, len(jobs)))()
        keep, outs = [], []
        for k, (ev, genes) in enumerate(jobs):
            g = np.ascontiguousarray(genes, np.int32)
            out = np.zeros(g.shape[0], CF_DTYPE)
            keep.append(g)
            outs.append(out)
            arr[k] = Job(ev.handle.value, g.shape[0], g.ctypes.data, out.ctypes.data)
        _check(self.lib.fxe_batch_eval_genes(self.handle, arr, len(jobs)))
        return outs

    def eval_genes_device(self, jobs, stream: int = 0):
        """jobs: [(GPUEvaluator, n, device genes pointer, device records pointer), ...]; not waited for."""
        arr = (Job * max(1, len(jobs)))()
        for k, (ev, n, dg, do) in enumerate(jobs):
            arr[k] = Job(ev.handle.value, int(n), int(dg), int(do))
        _check(self.lib.fxe_batch_eval_genes_device(self.handle, arr, len(jobs),
                                                    C.c_void_p(stream) if stream else None))

    def take_launches(self) -> int:
        n = C.c_int64(0)
        _check(self.lib.fxe_batch_take_launches(self.handle, C.byref(n)))
        return int(n.value)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.fxe_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GAJob(C.Structure):
    _fields_ = [("ctx", C.c_void_p), ("population", C.c_int32), ("generations", C.c_int32),
                ("cross_rate", C.c_double), ("mut_rate", C.c_double), ("seed", C.c_uint64),
                ("n_new", C.c_int32), ("steady", C.c_int32), ("intragenes", C.c_int32),
                ("adaptive", C.c_int32), ("k", C.c_double * 4), ("duplicates", C.c_int32),
                ("fitness", C.c_int32), ("sharing_alpha", C.c_double), ("sharing_peaks", C.c_double),
                ("sharing_scale", C.c_double), ("entropy_weight", C.c_double),
                ("temperature", C.c_double)]


FITNESS_MODELS = {"PSHARE": 0, "LINEAR": 1, "SMFREE": 2}


class GAEngine:
    """Docking jobs' genetic algorithms on the device (fxe_ga_*): admit, step, collect."""

    def __init__(self, max_jobs: int, precision: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        _check(self.lib.fxe_ga_create(int(max_jobs), int(precision), C.byref(h)))
        self.handle = h
        self.jobs = {}

    @staticmethod
    def job(ev: GPUEvaluator, population: int, generations: int, seed: int,
            cross_rate: float = 0.8, mut_rate: float = 0.03, n_new: int = 0, steady: bool = False,
            intragenes: bool = False, adaptive: bool = False, k=(1.0, 0.5, 1.0, 0.5),
            duplicates: bool = False, fitness: str = "PSHARE", sharing_alpha: float = 1.0,
            sharing_peaks: float = 5.0, sharing_scale: float = 10.0, entropy_weight: float = 0.5,
            temperature: float = 300.0) -> GAJob:
        """Defaults follow the reference's: crossover 0.8, mutation 0.03, PSHARE fitness, BOOM
        with boom_fraction 1, crossover at gene boundaries, fixed probabilities, duplicate
        chromosomes rejected (LIB/config_parser.cpp:108, 125-162)."""
        return GAJob(ev.handle.value, int(population), int(generations), float(cross_rate),
                     float(mut_rate), int(seed) & 0xFFFFFFFFFFFFFFFF, int(n_new), int(bool(steady)),
                     int(bool(intragenes)), int(bool(adaptive)), (C.c_double * 4)(*k),
                     int(bool(duplicates)), FITNESS_MODELS[fitness], float(sharing_alpha),
                     float(sharing_peaks), float(sharing_scale), float(entropy_weight),
                     float(temperature))

    def job_bytes(self, job: GAJob) -> int:
        b = C.c_int64(0)
        _check(self.lib.fxe_ga_job_bytes(C.byref(job), C.byref(b)))
        return int(b.value)

    def admit(self, job: GAJob, ev: GPUEvaluator) -> int:
        slot = C.c_int32(-1)
        _check(self.lib.fxe_ga_admit(self.handle, C.byref(job), C.byref(slot)))
        self.jobs[slot.value] = ev
        return slot.value

    def step(self):
        _check(self.lib.fxe_ga_step(self.handle))

    def finished(self) -> list:
        cap = max(1, len(self.jobs))
        out = np.zeros(cap, np.int32)
        n = C.c_int32(0)
        _check(self.lib.fxe_ga_finished(self.handle, ptr(out, _i), cap, C.byref(n)))
        return out[:n.value].tolist()

    def duplicates(self, slot: int):
        """(rejected, forced): candidates dropped as duplicates, and duplicates let through."""
        a, b = C.c_int64(0), C.c_int64(0)
        _check(self.lib.fxe_ga_duplicates(self.handle, int(slot), C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    def read_population(self, slot: int, population: int):
        ev = self.jobs[slot]
        g = np.zeros((population, ev.desc.n_genes), np.int32)
        e = np.zeros(population, np.float64)
        _check(self.lib.fxe_ga_population(self.handle, slot, ptr(g, _i), ptr(e, _d)))
        return g, e

    def ensemble(self, slot: int):
        """A finished job's ensemble, best first (the input of GPUEvaluator.cluster as the
        reference's cluster() receives chrom_snapshot): (ic (n, n_genes), energies (n,)). Call
        before collect."""
        ng = self.jobs[slot].desc.n_genes
        n = C.c_int64(0)
        _check(self.lib.fxe_ga_ensemble(self.handle, slot, 0, None, None, C.byref(n)))
        ic = np.zeros((n.value, ng), np.float64)
        e = np.zeros(n.value, np.float64)
        _check(self.lib.fxe_ga_ensemble(self.handle, slot, n.value, ptr(ic, _d), ptr(e, _d), C.byref(n)))
        return ic, e

    def collect(self, slot: int, temperature: float = 300.0):
        ev = self.jobs.pop(slot)
        g = np.zeros(ev.desc.n_genes, np.int32)
        be = C.c_double(0.0)
        t = Thermo()
        n = C.c_int64(0)
        _check(self.lib.fxe_ga_collect(self.handle, slot, float(temperature), ptr(g, _i), C.byref(be), C.byref(t),
                                       C.byref(n)))
        th = {k: getattr(t, k) for k, _ in Thermo._fields_}
        th["n_ensemble"] = int(n.value)
        return g, be.value, th

    def take_launches(self):
        a, b = C.c_int64(0), C.c_int64(0)
        _check(self.lib.fxe_ga_take_launches(self.handle, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.fxe_ga_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_lookup(precision: int, scored_atoms: int, poses: int) -> int:
    """The occupancy cap the autotuner's table holds for a size class (0: not tuned)."""
    b = C.c_int32(0)
    _check(load_library().fxe_autotune_lookup(int(precision), int(scored_atoms), int(poses), C.byref(b)))
    return int(b.value)


def ga_draws_per_pair(n_genes: int) -> int:
    """FXE_GA_DRAWS_PER_PAIR: the length of one pair's row of draws."""
    return 7 + 2 * int(n_genes) * 33


def ga_breed_draws(pop, fitness, draws, cross_rate, mut_rate, order=None, gene_prob=None,
                   intragenes=False, adaptive=False, k=(1.0, 0.5, 1.0, 0.5)) -> dict:
    """The GA engine's breeding on the device with the caller's draws (fxe_ga_breed_draws):
    draws is (n_pairs, ga_draws_per_pair(ng)). Returns children (2 n_pairs, ng) as uint32,
    draws used per pair and fitness_stats (total, max, mean)."""
    lib = load_library()
    pop = np.ascontiguousarray(np.asarray(pop, np.int64).astype(np.uint32).astype(np.int32))
    P, ng = pop.shape
    fit = np.ascontiguousarray(fitness, np.float64)
    draws = np.ascontiguousarray(draws, np.float64).reshape(-1, ga_draws_per_pair(ng))
    n_pairs = draws.shape[0]
    ordr = None if order is None else np.ascontiguousarray(order, np.int32)
    prob = None if gene_prob is None else np.ascontiguousarray(gene_prob, np.float32)
    kk = np.ascontiguousarray(k, np.float64)
    children = np.zeros((2 * max(n_pairs, 1), ng), np.int32)
    used = np.zeros(max(n_pairs, 1), np.int32)
    st = np.zeros(3, np.float64)
    _check(lib.fxe_ga_breed_draws(P, ng, ptr(pop, _i), ptr(fit, _d), ptr(ordr, _i) if ordr is not None else None,
                                  ptr(prob, _f) if prob is not None else None, float(cross_rate), float(mut_rate),
                                  int(bool(intragenes)), int(bool(adaptive)), ptr(kk, _d), n_pairs, ptr(draws, _d),
                                  ptr(children, _i), ptr(used, _i), ptr(st, _d)))
    return {"children": children[:2 * n_pairs].astype(np.int64) & 0xFFFFFFFF, "draws_used": used[:n_pairs],
            "total": float(st[0]), "max": float(st[1]), "mean": float(st[2])}


def ga_niche_counts(ic, sig_share: float, alpha: float = 1.0) -> np.ndarray:
    """PSHARE niche counts of a population given as ICs, on the device (fxe_ga_niche_counts)."""
    lib = load_library()
    ic = np.ascontiguousarray(ic, np.float64)
    out = np.empty(ic.shape[0], np.float64)
    _check(lib.fxe_ga_niche_counts(ic.shape[0], ic.shape[1], ptr(ic, _d), float(sig_share), float(alpha), ptr(out, _d)))
    return out


def ensemble_dedup(ic, energies) -> dict:
    """The statmech ensemble of chromosomes given as ICs, on the device (fxe_ensemble_dedup):
    sorted by energy, near-duplicates within 0.1 on every gene of the last one kept removed.
    Returns the kept input indices and energies, in energy order."""
    lib = load_library()
    ic = np.ascontiguousarray(ic, np.float64)
    e = np.ascontiguousarray(energies, np.float64)
    n = e.shape[0]
    ic = ic.reshape(n, -1)
    idx = np.zeros(max(n, 1), np.int64)
    ke = np.zeros(max(n, 1), np.float64)
    cnt = C.c_int64()
    _check(lib.fxe_ensemble_dedup(n, ic.shape[1], ptr(ic, _d), ptr(e, _d),
                                  idx.ctypes.data_as(C.POINTER(C.c_int64)), ptr(ke, _d), C.byref(cnt)))
    return {"index": idx[:cnt.value], "energy": ke[:cnt.value]}


def cleft_grid(centers, radii, spacing: float, ori) -> tuple:
    """The cleft grid of one or more spheres and its ICs, generated on the device
    (fxe_cleft_grid): (points (M, 3) float32, ICs (M, 3) float32), grid entry 0 not included."""
    lib = load_library()
    c = np.ascontiguousarray(np.asarray(centers, np.float32).reshape(-1, 3))
    r = np.ascontiguousarray(np.asarray(radii, np.float32).reshape(-1))
    o = np.ascontiguousarray(np.asarray(ori, np.float32).reshape(3))
    n = C.c_int64()
    rc = lib.fxe_cleft_grid(c.shape[0], ptr(c, _f), ptr(r, _f), float(spacing), ptr(o, _f), 0, None, None, C.byref(n))
    if rc not in (0, 6):      # FXE_ERR_CAPACITY: sized
        _check(rc)
    xyz = np.zeros((max(n.value, 1), 3), np.float32)
    ic = np.zeros((max(n.value, 1), 3), np.float32)
    _check(lib.fxe_cleft_grid(c.shape[0], ptr(c, _f), ptr(r, _f), float(spacing), ptr(o, _f), n.value,
                              ptr(xyz, _f), ptr(ic, _f), C.byref(n)))
    return xyz[:n.value], ic[:n.value]


def ic2cf(evaluator: GPUEvaluator, icv) -> np.void:
    """Scores one pose from its IC vector, as ic2cf(FA, VC, atoms, residue, cleftgrid, npar, icv)."""
    return evaluator.eval_ic(np.asarray(icv, np.float64)[None, :])[0]


def thermo(energies, multiplicity=None, temperature=300.0) -> dict:
    lib = load_library()
    e = np.ascontiguousarray(energies, np.float64)
    m = None if multiplicity is None else np.ascontiguousarray(multiplicity, np.int32)
    t = Thermo()
    _check(lib.fxe_thermo_compute(ptr(e, _d), ptr(m, _i) if m is not None else None, e.shape[0],
                                  float(temperature), C.byref(t)))
    return {k: getattr(t, k) for k, _ in Thermo._fields_}


def boltzmann_weights(energies, multiplicity=None, temperature=300.0) -> np.ndarray:
    lib = load_library()
    e = np.ascontiguousarray(energies, np.float64)
    m = None if multiplicity is None else np.ascontiguousarray(multiplicity, np.int32)
    w = np.zeros_like(e)
    _check(lib.fxe_thermo_weights(ptr(e, _d), ptr(m, _i) if m is not None else None, e.shape[0],
                                  float(temperature), ptr(w, _d)))
    return w


class StatMechEngine:
    """Canonical ensemble over docking poses (LIB/statmech.h:67-135), reduced on the GPU."""

    kB_kcal = 0.001987206   # LIB/statmech.h:26

    def __init__(self, temperature_K: float):
        self.T = float(temperature_K)
        self.beta = 1.0 / (self.kB_kcal * self.T)
        self._e: list[float] = []
        self._n: list[int] = []

    def add_sample(self, energy: float, multiplicity: int = 1):
        self._e.append(float(energy))
        self._n.append(int(multiplicity))

    def size(self) -> int:
        return len(self._e)

    def clear(self):
        self._e.clear()
        self._n.clear()

    def compute(self) -> dict:
        if not self._e:
            raise RuntimeError("StatMechEngine::compute: empty ensemble")
        return thermo(np.asarray(self._e), np.asarray(self._n, np.int32), self.T)

    def boltzmann_weights(self) -> np.ndarray:
        if not self._e:
            return np.zeros(0)
        return boltzmann_weights(np.asarray(self._e), np.asarray(self._n, np.int32), self.T)

    def delta_G(self, reference: "StatMechEngine") -> float:
        kT = self.kB_kcal * self.T
        return -kT * (self.compute()["log_Z"] - reference.compute()["log_Z"])

    @staticmethod
    def helmholtz(energies, temperature_K: float) -> float:
        return thermo(np.asarray(energies, np.float64), None, temperature_K)["free_energy"]
