"""ctypes mirror of include/fxe.h and packing of ``Descriptor`` into its structs."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .system import Descriptor

_f = C.POINTER(C.c_float)
_i = C.POINTER(C.c_int32)
_d = C.POINTER(C.c_double)
_b = C.POINTER(C.c_int8)

FXE_OK = 0
STATUS_NAMES = {0: "FXE_OK", 1: "FXE_ERR_INVALID_ARGS", 2: "FXE_ERR_ALLOC", 3: "FXE_ERR_LAUNCH",
                4: "FXE_ERR_TIMEOUT", 5: "FXE_ERR_OVER_BUDGET", 6: "FXE_ERR_CAPACITY",
                7: "FXE_ERR_NO_DEVICE", 8: "FXE_ERR_INTERNAL"}

POSE_SCORED, POSE_POLYHEDRON_FAILED, POSE_CLASHED, POSE_CAPACITY = 0, 1, 2, 3


class FlexResidue(C.Structure):
    _fields_ = [("first", C.c_int32), ("n_atoms", C.c_int32), ("n_rot", C.c_int32),
                ("backbone", _b), ("rot_xyz", _f), ("bonded", _b), ("prob", C.c_float)]


class ReceptorDesc(C.Structure):
    _fields_ = [("n_atoms", C.c_int32), ("xyz", _f), ("radius", _f), ("type", _i),
                ("ori", C.c_float * 3), ("globalmin", C.c_float * 3), ("globalmax", C.c_float * 3),
                ("maxwidth", C.c_float), ("n_grid", C.c_int32), ("grid_ic", _f),
                ("n_flex", C.c_int32), ("flex", C.POINTER(FlexResidue))]


class LigandDesc(C.Structure):
    _fields_ = [("n_atoms", C.c_int32), ("radius", _f), ("type", _i), ("rec", _i), ("shift", _f),
                ("ic", _f), ("n_build", C.c_int32), ("build_order", _i), ("bonded", _b),
                ("n_genes", C.c_int32), ("gene_type", _i), ("gene_atom", _i), ("gene_min", _d),
                ("gene_max", _d), ("gene_del", _d), ("gene_map", _i)]


class EmatDesc(C.Structure):
    _fields_ = [("ntypes", C.c_int32), ("weight", _i), ("offset", _i), ("x", _f), ("y", _f)]


class Params(C.Structure):
    _fields_ = [("permeability", C.c_float), ("dee_clash", C.c_float),
                ("intramolecular", C.c_int32), ("solventterm", C.c_float)]


class CF(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("com", "con", "wal", "sas", "elec", "gist", "hbond",
                                          "gist_desolv", "metal_coord", "totsas", "evalue")] + \
               [("rclash", C.c_int32), ("status", C.c_int32)]


class Thermo(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("temperature", "log_Z", "free_energy", "mean_energy",
                                          "mean_energy_sq", "heat_capacity", "entropy",
                                          "std_energy")]


CF_DTYPE = np.dtype([(k, np.float64) for k in ("com", "con", "wal", "sas", "elec", "gist",
                                               "hbond", "gist_desolv", "metal_coord", "totsas",
                                               "evalue")] + [("rclash", np.int32),
                                                             ("status", np.int32)])
assert CF_DTYPE.itemsize == C.sizeof(CF)


def ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


class Packed:
    """A Descriptor packed into the C structs, holding the arrays the pointers refer to."""

    def __init__(self, d: Descriptor):
        self.keep = []

        def k(a, dt):
            a = np.ascontiguousarray(a, dt)
            self.keep.append(a)
            return a

        r = ReceptorDesc()
        r.n_atoms = d.n_rec
        r.xyz = ptr(k(d.rec_xyz, np.float32), _f)
        r.radius = ptr(k(d.rec_radius, np.float32), _f)
        r.type = ptr(k(d.rec_type, np.int32), _i)
        r.ori[:] = [float(x) for x in d.ori]
        r.globalmin[:] = [float(x) for x in d.globalmin]
        r.globalmax[:] = [float(x) for x in d.globalmax]
        r.maxwidth = d.maxwidth
        r.n_grid = d.grid_ic.shape[0]
        r.grid_ic = ptr(k(d.grid_ic, np.float32), _f)
        r.n_flex = d.n_flex
        if d.n_flex:
            fr = (FlexResidue * d.n_flex)()
            a0 = r0 = b0 = 0
            for i in range(d.n_flex):
                na, nr = int(d.flex_natm[i]), int(d.flex_nrot[i])
                fr[i].first = int(d.flex_first[i])
                fr[i].n_atoms = na
                fr[i].n_rot = nr
                fr[i].backbone = ptr(k(d.flex_isbb[a0:a0 + na], np.int8), _b)
                fr[i].rot_xyz = ptr(k(d.flex_xyz[r0:r0 + nr * na], np.float32), _f)
                fr[i].bonded = ptr(k(d.flex_bonded[b0:b0 + na * na], np.int8), _b)
                fr[i].prob = float(d.flex_prob[i])
                a0, r0, b0 = a0 + na, r0 + nr * na, b0 + na * na
            self.keep.append(fr)
            r.flex = fr
        lg = LigandDesc()
        lg.n_atoms = d.n_lig
        lg.radius = ptr(k(d.lig_radius, np.float32), _f)
        lg.type = ptr(k(d.lig_type, np.int32), _i)
        lg.rec = ptr(k(d.lig_rec, np.int32), _i)
        lg.shift = ptr(k(d.lig_shift, np.float32), _f)
        lg.ic = ptr(k(d.lig_ic, np.float32), _f)
        lg.n_build = d.build_order.shape[0]
        lg.build_order = ptr(k(d.build_order, np.int32), _i)
        lg.bonded = ptr(k(d.bonded, np.int8), _b)
        lg.n_genes = d.n_genes
        lg.gene_type = ptr(k(d.gene_typ, np.int32), _i)
        lg.gene_atom = ptr(k(d.gene_atm, np.int32), _i)
        lg.gene_min = ptr(k(d.gene_min, np.float64), _d)
        lg.gene_max = ptr(k(d.gene_max, np.float64), _d)
        lg.gene_del = ptr(k(d.gene_del, np.float64), _d)
        lg.gene_map = ptr(k(d.gene_map, np.int32), _i)
        e = EmatDesc()
        e.ntypes = d.ntypes
        e.weight = ptr(k(d.emat_weight, np.int32), _i)
        e.offset = ptr(k(d.emat_off, np.int32), _i)
        e.x = ptr(k(d.emat_x, np.float32), _f)
        e.y = ptr(k(d.emat_y, np.float32), _f)
        p = Params()
        p.permeability = d.permeability
        p.dee_clash = d.dee_clash
        p.intramolecular = d.intramolecular
        p.solventterm = d.solventterm
        self.rec, self.lig, self.emat, self.params = r, lg, e, p
