"""ctypes driver for the C restatement (oracle/_build/libfxe_oracle.so).

TEST INFRASTRUCTURE ONLY: the checker for the GPU path (tests/, smoke check, the bench's
CPU-baseline leg). ``build()`` compiles it from oracle/fxe_oracle.c with the Makefile here.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from flexaidds_gb300.capi import CF, CF_DTYPE, Packed, Thermo, _d, _f, _i, ptr
from flexaidds_gb300.system import Descriptor

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libfxe_oracle.so")
_lib = None


class Contact(C.Structure):
    _fields_ = [("pose", C.c_int32), ("atom", C.c_int32), ("partner", C.c_int32),
                ("area", C.c_float), ("dist", C.c_float)]


CONTACT_DTYPE = np.dtype([("pose", np.int32), ("atom", np.int32), ("partner", np.int32),
                          ("area", np.float32), ("dist", np.float32)])


class Counts(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("atoms", "candidates", "contacts", "edges", "arc_edges",
                                         "triangles", "vertices", "built_atoms", "no_partner",
                                         "plane_tests")]


def build():
    subprocess.run(["make", "-s", "-C", _HERE, "port"], check=True)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _lib.fxo_eval_ic.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, _d,
                                     C.c_void_p, _f, C.c_void_p, C.c_int64,
                                     C.POINTER(C.c_int64), C.c_void_p]
        _lib.fxo_genes_to_ic.argtypes = [C.c_void_p, C.c_int32, _i, _d]
        _lib.fxo_thermo.argtypes = [_d, _i, C.c_int64, C.c_double, C.c_void_p]
        _lib.fxo_thermo_weights.argtypes = [_d, _i, C.c_int64, C.c_double, _d]
        _lib.fxo_set_reference_compat.argtypes = [C.c_int]
        _lib.fxo_set_trig_rounding.argtypes = [C.c_int]
        _lib.fxo_solve_3x3.argtypes = [_d, _d, _d, _d]
        _lib.fxo_solve_2xS.argtypes = [_d, _d, C.c_float, _d, _d]
        _lib.fxo_cosPQR.argtypes = [_d, _d, _d]
        _lib.fxo_cosPQR.restype = C.c_double
        _lib.fxo_spherical_arc.argtypes = [_d, C.c_double, _d, C.c_double, _d, C.c_double, C.c_float]
        _lib.fxo_spherical_arc.restype = C.c_double
        _lib.fxo_build_ic.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, _d, _f]
        _lib.fxo_cluster.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, _d, _d, C.c_int32, C.c_float,
                                     C.c_int32, _i, _i, _d, _d, _i, _f, _f, _i]
    return _lib


def lib():
    return _load()


class Oracle:
    """Scores poses of one Descriptor with the C restatement."""

    def __init__(self, d: Descriptor):
        self.d = d
        self.packed = Packed(d)

    def eval_ic(self, ic: np.ndarray, want_xyz=False, want_contacts=False, counts=False):
        lib = _load()
        ic = np.ascontiguousarray(ic, np.float64)
        n = ic.shape[0]
        out = np.zeros(n, CF_DTYPE)
        xyz = np.zeros((n, self.d.n_lig, 3), np.float32) if want_xyz else None
        cap = n * self.d.n_lig * 128 if want_contacts else 0
        cont = np.zeros(max(cap, 1), CONTACT_DTYPE)
        ncont = C.c_int64(0)
        cnt = Counts() if counts else None
        pk = self.packed
        rc = lib.fxo_eval_ic(C.byref(pk.rec), C.byref(pk.lig), C.byref(pk.emat), C.byref(pk.params),
                             n, ptr(ic, _d), out.ctypes.data_as(C.c_void_p),
                             ptr(xyz, _f) if want_xyz else None,
                             cont.ctypes.data_as(C.c_void_p) if want_contacts else None, cap,
                             C.byref(ncont), C.byref(cnt) if counts else None)
        if rc != 0:
            raise RuntimeError(f"fxo_eval_ic failed ({rc})")
        res = {"cf": out}
        if want_xyz:
            res["xyz"] = xyz
        if want_contacts:
            res["contacts"] = cont[:min(ncont.value, cap)].copy()
        if counts:
            res["counts"] = {k: getattr(cnt, k) for k, _ in Counts._fields_}
        return res

    def build_ic(self, ic: np.ndarray) -> np.ndarray:
        """Ligand coordinates (n, n_lig, 3) as calc_rmsd_chrom builds them."""
        lib = _load()
        ic = np.ascontiguousarray(ic, np.float64)
        xyz = np.zeros((ic.shape[0], self.d.n_lig, 3), np.float32)
        if lib.fxo_build_ic(C.byref(self.packed.rec), C.byref(self.packed.lig), ic.shape[0], ptr(ic, _d),
                            ptr(xyz, _f)) != 0:
            raise RuntimeError("fxo_build_ic failed")
        return xyz

    def cluster(self, ic: np.ndarray, app_evalue: np.ndarray, temperature: int = 0, rmsd: float = 2.0,
                max_results: int = 10) -> dict:
        """CF-based clustering, serial restatement of cluster (LIB/cluster.cpp)."""
        lib = _load()
        ic = np.ascontiguousarray(ic, np.float64)
        e = np.ascontiguousarray(app_evalue, np.float64)
        n, R = ic.shape[0], int(max_results)
        top, freq = np.zeros(R, np.int32), np.zeros(R, np.int32)
        tcf, acf = np.zeros(R, np.float64), np.zeros(R, np.float64)
        member, rms = np.zeros(n, np.int32), np.zeros(n, np.float32)
        top_rmsd = np.zeros((R, R), np.float32)
        nc = C.c_int32(0)
        rc = lib.fxo_cluster(C.byref(self.packed.rec), C.byref(self.packed.lig), n, ptr(ic, _d), ptr(e, _d),
                             int(temperature), float(rmsd), R, ptr(top, _i), ptr(freq, _i), ptr(tcf, _d),
                             ptr(acf, _d), ptr(member, _i), ptr(rms, _f), ptr(top_rmsd, _f), C.byref(nc))
        if rc != 0:
            raise RuntimeError(f"fxo_cluster failed ({rc})")
        return {"n_clusters": nc.value, "top": top, "freq": freq, "tcf": tcf, "acf": acf,
                "member_of": member, "rmsd": rms, "top_rmsd": top_rmsd}

    def genes_to_ic(self, genes: np.ndarray) -> np.ndarray:
        lib = _load()
        genes = np.ascontiguousarray(genes, np.int32)
        ic = np.zeros(genes.shape, np.float64)
        lib.fxo_genes_to_ic(C.byref(self.packed.lig), genes.shape[0], ptr(genes, _i), ptr(ic, _d))
        return ic


def set_reference_compat(on: bool):
    """Replays the reference's stale-slot read in order_faces (for pinning against it)."""
    _load().fxo_set_reference_compat(1 if on else 0)


def set_trig_rounding(correctly_rounded: bool):
    """Pose-build trigonometry: the C library's cosf/sinf (False, as the reference) or the
    correctly rounded values the CUDA build kernel computes (True)."""
    _load().fxo_set_trig_rounding(1 if correctly_rounded else 0)


def thermo(e, mult=None, temperature=300.0) -> dict:
    lib = _load()
    e = np.ascontiguousarray(e, np.float64)
    m = None if mult is None else np.ascontiguousarray(mult, np.int32)
    t = Thermo()
    rc = lib.fxo_thermo(ptr(e, _d), ptr(m, _i) if m is not None else None, e.shape[0],
                        temperature, C.byref(t))
    if rc != 0:
        raise ValueError("invalid ensemble")
    return {k: getattr(t, k) for k, _ in Thermo._fields_}


def thermo_weights(e, mult=None, temperature=300.0) -> np.ndarray:
    lib = _load()
    e = np.ascontiguousarray(e, np.float64)
    m = None if mult is None else np.ascontiguousarray(mult, np.int32)
    w = np.zeros_like(e)
    rc = lib.fxo_thermo_weights(ptr(e, _d), ptr(m, _i) if m is not None else None, e.shape[0],
                                temperature, ptr(w, _d))
    if rc != 0:
        raise ValueError("invalid ensemble")
    return w
