"""ctypes driver for the reference's own scoring chain (oracle/_ref/libfxe_ref.so).

TEST INFRASTRUCTURE ONLY: used by tests/ and by the fixture generator to produce the expected
values; never by the product. The library exists only where the reference checkout was present
at build time (``make -C oracle ref``); ``available()`` says whether it does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from flexaidds_gb300.system import Descriptor, SystemInputs

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libfxe_ref.so")
# the reference checkout (its sources build oracle/_ref; its data files are read by some tests)
REFERENCE_ROOT = os.environ.get("FXE_REFERENCE_ROOT", "/root/reference")
_lib = None

_f = C.POINTER(C.c_float)
_i = C.POINTER(C.c_int32)
_d = C.POINTER(C.c_double)
_b = C.POINTER(C.c_int8)


class RefInput(C.Structure):
    _fields_ = [
        ("n_rec", C.c_int32), ("rec_xyz", _f), ("rec_type", _i), ("rec_radius", _f),
        ("n_lig", C.c_int32), ("lig_xyz", _f), ("lig_type", _i), ("lig_radius", _f),
        ("n_bonds", C.c_int32), ("bonds", _i), ("lig_rec", _i), ("gpa", C.c_int32 * 3),
        ("n_flex", C.c_int32), ("flex", _i), ("n_grid", C.c_int32), ("grid_xyz", _f),
        ("ntypes", C.c_int32), ("emat_weight", _i), ("emat_off", _i), ("emat_x", _f),
        ("emat_y", _f), ("permeability", C.c_float), ("dee_clash", C.c_float),
        ("intramolecular", C.c_int32), ("solventterm", C.c_float),
        ("n_flexres", C.c_int32), ("flex_first", _i), ("flex_natm", _i), ("flex_nrot", _i),
        ("flex_isbb", _b), ("flex_xyz", _f), ("flex_nbonds", _i), ("flex_bonds", _i),
    ]


class RefSizes(C.Structure):
    _fields_ = [("n_atoms", C.c_int32), ("n_lig", C.c_int32), ("n_genes", C.c_int32),
                ("n_grid", C.c_int32), ("n_mov", C.c_int32)]


def available() -> bool:
    return os.path.exists(LIB_PATH)


def _load():
    global _lib
    if _lib is None:
        if not available():
            raise FileNotFoundError(f"{LIB_PATH} not built (make -C oracle ref)")
        _lib = C.CDLL(LIB_PATH)
        _lib.ref_setup.argtypes = [C.POINTER(RefInput)]
        _lib.ref_sizes.argtypes = [C.POINTER(RefSizes)]
        _lib.ref_export.argtypes = [_f, _f, _f, _f, _f, _f, _f, _i, _i, _b, _i, _i, _d, _d, _d, _i, _d]
        _lib.ref_eval.argtypes = [C.c_int32, _d, _d, _i, _f]
        _lib.ref_last_contacts.argtypes = [C.c_int32, C.c_int32, _i, _d, _d]
        _lib.ref_export_flex_bonded.argtypes = [_b]
        _lib.ref_cluster.argtypes = [C.c_int32, _d, _d, C.c_int32, C.c_float, C.c_int32, C.c_char_p]
        _lib.ref_adapter_pack.argtypes = [_i, C.c_char_p, C.c_int32]
        _lib.ref_adapter_get.argtypes = [C.c_char_p, C.c_void_p]
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


class RefHarness:
    """One reference scoring state (the harness keeps a single global state)."""

    def __init__(self, inp: SystemInputs):
        lib = _load()
        self.inp = inp
        rec, lig = inp.receptor, inp.ligand
        self._keep = []

        def keep(a, dt):
            a = np.ascontiguousarray(a, dt)
            self._keep.append(a)
            return a

        bonds = keep(np.asarray(lig.bonds, np.int32).reshape(-1), np.int32)
        flex = np.full((max(1, len(lig.flex)), 3), -1, np.int32)
        for j, atoms in enumerate(lig.flex):
            flex[j, :len(atoms)] = atoms
        flex = keep(flex, np.int32)
        w, off, ex, ey = inp.emat_tables()
        r = RefInput()
        r.n_rec = rec.xyz.shape[0]
        r.rec_xyz = _p(keep(rec.xyz, np.float32), _f)
        r.rec_type = _p(keep(rec.type, np.int32), _i)
        r.rec_radius = _p(keep(rec.radius, np.float32), _f)
        r.n_lig = lig.xyz.shape[0]
        r.lig_xyz = _p(keep(lig.xyz, np.float32), _f)
        r.lig_type = _p(keep(lig.type, np.int32), _i)
        r.lig_radius = _p(keep(lig.radius, np.float32), _f)
        r.n_bonds = len(lig.bonds)
        r.bonds = _p(bonds, _i)
        r.lig_rec = _p(keep(lig.rec, np.int32), _i)
        r.gpa[:] = list(lig.gpa)
        r.n_flex = len(lig.flex)
        r.flex = _p(flex, _i)
        r.n_grid = inp.grid_xyz.shape[0]
        r.grid_xyz = _p(keep(inp.grid_xyz, np.float32), _f)
        r.ntypes = inp.emat.shape[0]
        r.emat_weight = _p(keep(w, np.int32), _i)
        r.emat_off = _p(keep(off, np.int32), _i)
        r.emat_x = _p(keep(ex, np.float32), _f)
        r.emat_y = _p(keep(ey, np.float32), _f)
        r.permeability = inp.permeability
        r.dee_clash = inp.dee_clash
        r.intramolecular = inp.intramolecular
        r.solventterm = inp.solventterm
        fl = rec.flex
        r.n_flexres = len(fl)
        if fl:
            r.flex_first = _p(keep([f.first for f in fl], np.int32), _i)
            r.flex_natm = _p(keep([f.natm for f in fl], np.int32), _i)
            r.flex_nrot = _p(keep([f.n_rot for f in fl], np.int32), _i)
            r.flex_isbb = _p(keep(np.concatenate([f.isbb for f in fl]), np.int8), _b)
            r.flex_xyz = _p(keep(np.concatenate([f.rot_xyz.reshape(-1) for f in fl]), np.float32), _f)
            r.flex_nbonds = _p(keep([len(f.bonds) for f in fl], np.int32), _i)
            r.flex_bonds = _p(keep(np.asarray([b for f in fl for b in f.bonds], np.int32).reshape(-1),
                                   np.int32), _i)
        self._r = r
        if lib.ref_setup(C.byref(r)) != 0:
            raise RuntimeError("reference set-up failed")
        s = RefSizes()
        lib.ref_sizes(C.byref(s))
        self.sizes = s

    def descriptor(self) -> Descriptor:
        lib = _load()
        s = self.sizes
        n, ng = s.n_lig, s.n_genes
        ori = np.zeros(3, np.float32)
        gmin = np.zeros(3, np.float32)
        gmax = np.zeros(3, np.float32)
        mw = np.zeros(1, np.float32)
        grid_ic = np.zeros((s.n_grid, 3), np.float32)
        lig_ic = np.zeros((n, 3), np.float32)
        shift = np.zeros(n, np.float32)
        lrec = np.zeros((n, 4), np.int32)
        mov = np.zeros(s.n_mov, np.int32)
        bonded = np.zeros((n, n), np.int8)
        typ = np.zeros(ng, np.int32)
        atm = np.zeros(ng, np.int32)
        gmn = np.zeros(ng, np.float64)
        gmx = np.zeros(ng, np.float64)
        gdl = np.zeros(ng, np.float64)
        gmp = np.zeros(ng, np.int32)
        opt = np.zeros(ng, np.float64)
        lib.ref_export(_p(ori, _f), _p(gmin, _f), _p(gmax, _f), _p(mw, _f), _p(grid_ic, _f),
                       _p(lig_ic, _f), _p(shift, _f), _p(lrec, _i), _p(mov, _i), _p(bonded, _b),
                       _p(typ, _i), _p(atm, _i), _p(gmn, _d), _p(gmx, _d), _p(gdl, _d),
                       _p(gmp, _i), _p(opt, _d))
        w, off, ex, ey = self.inp.emat_tables()
        rec, lig = self.inp.receptor, self.inp.ligand
        fx = {}
        if rec.flex:
            fb = np.zeros(sum(f.natm * f.natm for f in rec.flex), np.int8)
            lib.ref_export_flex_bonded(_p(fb, _b))
            fx = dict(flex_first=np.asarray([f.first for f in rec.flex], np.int32),
                      flex_natm=np.asarray([f.natm for f in rec.flex], np.int32),
                      flex_nrot=np.asarray([f.n_rot for f in rec.flex], np.int32),
                      flex_isbb=np.concatenate([f.isbb for f in rec.flex]).astype(np.int8),
                      flex_xyz=np.concatenate([f.rot_xyz.reshape(-1, 3) for f in rec.flex]).astype(np.float32),
                      flex_bonded=fb, flex_prob=np.asarray([f.prob for f in rec.flex], np.float32))
        return Descriptor(**fx,
            rec_xyz=rec.xyz.copy(), rec_radius=rec.radius.copy(), rec_type=rec.type.copy(),
            ori=ori, globalmin=gmin, globalmax=gmax, maxwidth=float(mw[0]), grid_ic=grid_ic,
            lig_radius=lig.radius.copy(), lig_type=lig.type.copy(), lig_rec=lrec,
            lig_shift=shift, lig_ic=lig_ic, build_order=mov, bonded=bonded, gene_typ=typ,
            gene_atm=atm, gene_min=gmn, gene_max=gmx, gene_del=gdl, gene_map=gmp, opt_par=opt,
            ntypes=int(self.inp.emat.shape[0]), emat_weight=w, emat_off=off, emat_x=ex,
            emat_y=ey, permeability=self.inp.permeability, dee_clash=self.inp.dee_clash,
            intramolecular=self.inp.intramolecular, solventterm=self.inp.solventterm)

    def adapter_arrays(self) -> dict:
        """What the product's C++ adapter (flexaidds_gb300/adapter/fxe_flexaid_pack.cpp) packs from
        this harness's reference state, by descriptor field name."""
        lib = _load()
        sz = np.zeros(7, np.int32)
        msg = C.create_string_buffer(512)
        if lib.ref_adapter_pack(_p(sz, _i), msg, 512) != 0:
            raise RuntimeError(msg.value.decode())
        n_rec, n_grid, n, ng, n_build, n_pts, n_flex = (int(x) for x in sz)
        spec = {"rec_xyz": (n_rec * 3, np.float32), "rec_radius": (n_rec, np.float32), "rec_type": (n_rec, np.int32),
                "grid_ic": (n_grid * 3, np.float32), "lig_radius": (n, np.float32), "lig_type": (n, np.int32),
                "lig_rec": (n * 4, np.int32), "lig_shift": (n, np.float32), "lig_ic": (n * 3, np.float32),
                "build_order": (n_build, np.int32), "bonded": (n * n, np.int8), "gene_typ": (ng, np.int32),
                "gene_atm": (ng, np.int32), "gene_min": (ng, np.float64), "gene_max": (ng, np.float64),
                "gene_del": (ng, np.float64), "gene_map": (ng, np.int32), "emat_x": (n_pts, np.float32),
                "emat_y": (n_pts, np.float32), "frame": (10, np.float32), "params": (4, np.float32),
                "flex_info": (4 * n_flex, np.int32)}
        t = int(self.inp.emat.shape[0])
        spec["emat_weight"] = (t * t, np.int32)
        spec["emat_off"] = (t * t + 1, np.int32)
        if n_flex:
            fl = self.inp.receptor.flex
            spec["flex_backbone"] = (sum(f.natm for f in fl), np.int8)
            spec["flex_xyz"] = (sum(f.natm * f.n_rot * 3 for f in fl), np.float32)
            spec["flex_bonded"] = (sum(f.natm * f.natm for f in fl), np.int8)
        out = {}
        for k, (cnt, dt) in spec.items():
            a = np.zeros(max(cnt, 1), dt)
            got = lib.ref_adapter_get(k.encode(), a.ctypes.data_as(C.c_void_p))
            if got != cnt:
                raise RuntimeError(f"adapter array {k}: {got} entries, expected {cnt}")
            out[k] = a[:cnt]
        return out

    def eval(self, ic: np.ndarray, want_xyz: bool = False):
        """Scores poses given as decoded ICs. Returns (cf[n, 11], status[n], xyz or None)."""
        lib = _load()
        ic = np.ascontiguousarray(ic, np.float64)
        n = ic.shape[0]
        cf = np.zeros((n, 11), np.float64)
        st = np.zeros(n, np.int32)
        xyz = np.zeros((n, self.sizes.n_lig, 3), np.float32) if want_xyz else None
        lib.ref_eval(n, _p(ic, _d), _p(cf, _d), _p(st, _i), _p(xyz, _f) if want_xyz else None)
        return cf, st, xyz

    def last_contacts(self):
        """Per scored atom (side-chain atoms, then the ligand): (partner Calc indices, areas,
        distances) of the last scored pose."""
        lib = _load()
        out = []
        cap = 4096
        n_sc = sum(int((f.isbb == 0).sum()) for f in self.inp.receptor.flex)
        for i in range(n_sc + self.sizes.n_lig):
            p = np.zeros(cap, np.int32)
            a = np.zeros(cap, np.float64)
            d = np.zeros(cap, np.float64)
            m = lib.ref_last_contacts(i, cap, _p(p, _i), _p(a, _d), _p(d, _d))
            out.append((p[:m].copy(), a[:m].copy(), d[:m].copy()))
        return out

    def cluster(self, ic: np.ndarray, app_evalue: np.ndarray, temperature: int, rmsd: float,
                max_results: int, prefix: str) -> str:
        """Runs the reference's CF-based clustering (cluster, LIB/cluster.cpp) and returns the
        text of the .cad file it writes at <prefix>.cad (its <prefix>_<k>.pdb files stay beside
        it)."""
        lib = _load()
        ic = np.ascontiguousarray(ic, np.float64)
        e = np.ascontiguousarray(app_evalue, np.float64)
        rc = lib.ref_cluster(ic.shape[0], _p(ic, _d), _p(e, _d), int(temperature), float(rmsd),
                             int(max_results), prefix.encode())
        if rc != 0:
            raise RuntimeError(f"ref_cluster failed ({rc})")
        with open(prefix + ".cad") as f:
            return f.read()
