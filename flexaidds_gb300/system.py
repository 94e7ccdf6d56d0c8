"""Docking-system descriptors: everything the evaluation path reads, as flat arrays.

A ``Descriptor`` is the packed form of the reference's set-up state for one receptor, one
ligand and one energy matrix (the FA / atoms / residue / cleft-grid / gene-limit data that
LIB/ic2cf.cpp, LIB/buildcc.cpp, LIB/vcfunction.cpp and LIB/Vcontacts.cpp read). It crosses the
C ABI as ``fxe_receptor_desc`` / ``fxe_ligand_desc`` / ``fxe_emat_desc`` (include/fxe.h).

Atom numbering follows the reference's ``Calc`` order (LIB/Vcontacts.cpp:1600-1630): receptor
atoms first in residue order, then the ligand atoms. Ligand-local indices are used inside the
ligand arrays, with -1 standing for the reference frame (``rec == 0`` in the reference).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import synth

# gene types (optmap.typ, LIB/flexaid.h:175-180 / LIB/ic2cf.cpp:56-105)
GENE_GRID = -1
GENE_DIS = 0
GENE_ANG = 1
GENE_DIH = 2
GENE_ROTAMER = 4


@dataclass
class SystemInputs:
    """Raw generator output for one docking system (no set-up applied yet)."""
    receptor: synth.Receptor
    ligand: synth.Ligand
    grid_xyz: np.ndarray                 # (M, 3) float32, cleft points (entry 0 not included)
    emat: np.ndarray                     # (T, T) float32 single values
    emat_weight: np.ndarray = None       # (T, T) int32, 1 = single value, 0 = density curve
    emat_curves: dict = None             # {(i, j): [(x, y), ...]} for density entries (0-based types)
    permeability: float = 1.0
    dee_clash: float = 0.5
    intramolecular: int = 1
    solventterm: float = 0.0

    def __post_init__(self):
        t = self.emat.shape[0]
        if self.emat_weight is None:
            self.emat_weight = np.ones((t, t), np.int32)
        if self.emat_curves is None:
            self.emat_curves = {}

    def emat_tables(self):
        """Flat (weight, offsets, x, y) arrays in the reference's energy_values layout."""
        t = self.emat.shape[0]
        off = [0]
        xs, ys = [], []
        for i in range(t):
            for j in range(t):
                if self.emat_weight[i, j]:
                    xs.append(-1.0)
                    ys.append(float(self.emat[i, j]))
                else:
                    pts = self.emat_curves[(min(i, j), max(i, j))]
                    for x, y in pts:
                        xs.append(float(x))
                        ys.append(float(y))
                off.append(len(xs))
        return (np.ascontiguousarray(self.emat_weight.reshape(-1), np.int32),
                np.asarray(off, np.int32), np.asarray(xs, np.float32), np.asarray(ys, np.float32))


@dataclass
class Descriptor:
    """Packed set-up state (the evaluation path's whole input besides the chromosomes)."""
    # receptor (Calc order)
    rec_xyz: np.ndarray
    rec_radius: np.ndarray
    rec_type: np.ndarray
    ori: np.ndarray
    globalmin: np.ndarray
    globalmax: np.ndarray
    maxwidth: float
    grid_ic: np.ndarray          # (n_grid, 3) dis, ang, dih; entry 0 = initial anchor
    # ligand
    lig_radius: np.ndarray
    lig_type: np.ndarray
    lig_rec: np.ndarray          # (n, 4) int32, -1 = reference frame / no cascade
    lig_shift: np.ndarray
    lig_ic: np.ndarray           # (n, 3) base dis, ang, dih
    build_order: np.ndarray      # (n_mov,) int32 (FA->mov[0])
    bonded: np.ndarray           # (n, n) int8
    gene_typ: np.ndarray
    gene_atm: np.ndarray
    gene_min: np.ndarray
    gene_max: np.ndarray
    gene_del: np.ndarray
    gene_map: np.ndarray
    opt_par: np.ndarray          # initial ICs
    # energy matrix
    ntypes: int
    emat_weight: np.ndarray
    emat_off: np.ndarray
    emat_x: np.ndarray
    emat_y: np.ndarray
    # scoring parameters
    permeability: float = 1.0
    dee_clash: float = 0.5
    intramolecular: int = 1
    solventterm: float = 0.0
    # flexible side chains (residues with rotamers), in Calc order; gene type 4 names the
    # residue by its index here
    flex_first: np.ndarray = None    # (R,) int32 receptor index of each residue's first atom
    flex_natm: np.ndarray = None     # (R,) int32
    flex_nrot: np.ndarray = None     # (R,) int32, rotamer 0 = the receptor's coordinates
    flex_isbb: np.ndarray = None     # (sum natm,) int8, 1 = backbone (not scored)
    flex_xyz: np.ndarray = None      # (sum nrot * natm, 3) float32
    flex_bonded: np.ndarray = None   # (sum natm * natm,) int8, residue.bonded
    flex_prob: np.ndarray = None     # (R,) float32, flxsc.prob (GA rotamer moves)
    decode: list = field(default_factory=list)

    def __post_init__(self):
        if self.flex_first is None:
            self.flex_first = np.zeros(0, np.int32)
            self.flex_natm = np.zeros(0, np.int32)
            self.flex_nrot = np.zeros(0, np.int32)
            self.flex_isbb = np.zeros(0, np.int8)
            self.flex_xyz = np.zeros((0, 3), np.float32)
            self.flex_bonded = np.zeros(0, np.int8)
        if self.flex_prob is None:
            self.flex_prob = np.ones(self.flex_first.shape[0], np.float32)

    @property
    def n_flex(self):
        return int(self.flex_first.shape[0])

    @property
    def n_sc(self):
        """Scored side-chain atoms (the non-backbone atoms of the flexible residues)."""
        return int((self.flex_isbb == 0).sum())

    @property
    def n_rec(self):
        return int(self.rec_xyz.shape[0])

    @property
    def n_lig(self):
        return int(self.lig_radius.shape[0])

    @property
    def n_genes(self):
        return int(self.gene_typ.shape[0])

    def decode_tables(self):
        """Cumulative-bin tables for genetoic, one per gene (see ``gene_bins``)."""
        if not self.decode:
            self.decode = [gene_bins(self.gene_min[g], self.gene_max[g], self.gene_del[g],
                                     int(self.gene_map[g])) for g in range(self.n_genes)]
        return self.decode

    _ARRAYS = ("rec_xyz", "rec_radius", "rec_type", "ori", "globalmin", "globalmax", "grid_ic",
               "lig_radius", "lig_type", "lig_rec", "lig_shift", "lig_ic", "build_order", "bonded",
               "gene_typ", "gene_atm", "gene_min", "gene_max", "gene_del", "gene_map", "opt_par",
               "emat_weight", "emat_off", "emat_x", "emat_y")
    _SCALARS = ("maxwidth", "ntypes", "permeability", "dee_clash", "intramolecular", "solventterm")
    _FLEX = ("flex_first", "flex_natm", "flex_nrot", "flex_isbb", "flex_xyz", "flex_bonded")

    def to_arrays(self, prefix: str = "") -> dict:
        """Flat name -> array mapping (for np.savez)."""
        out = {prefix + k: np.asarray(getattr(self, k)) for k in self._ARRAYS}
        out.update({prefix + k: np.asarray(getattr(self, k)) for k in self._SCALARS})
        if self.n_flex:
            out.update({prefix + k: np.asarray(getattr(self, k)) for k in self._FLEX + ("flex_prob",)})
        return out

    @classmethod
    def from_arrays(cls, arrs, prefix: str = "") -> "Descriptor":
        kw = {k: np.asarray(arrs[prefix + k]).copy() for k in cls._ARRAYS}
        if prefix + "flex_first" in arrs:
            kw.update({k: np.asarray(arrs[prefix + k]).copy() for k in cls._FLEX})
            if prefix + "flex_prob" in arrs:
                kw["flex_prob"] = np.asarray(arrs[prefix + "flex_prob"]).copy()
        for k in cls._SCALARS:
            v = np.asarray(arrs[prefix + k]).item()
            kw[k] = int(v) if k in ("ntypes", "intramolecular") else float(v)
        return cls(**kw)

    def genes_to_ic(self, genes: np.ndarray) -> np.ndarray:
        """Decode int32 genes to ICs exactly as LIB/gaboom.cpp:2887-2906 (genetoic) does."""
        genes = np.asarray(genes, np.int32)
        out = np.empty(genes.shape, np.float64)
        for g, tab in enumerate(self.decode_tables()):
            u = genes[..., g].astype(np.float64) / (2147483647.0 + 1.0)
            i = np.searchsorted(tab, u, side='left')
            out[..., g] = self.gene_min[g] + self.gene_del[g] * i.astype(np.float64)
        return out


def gene_bins(gmin: float, gmax: float, gdel: float, gmap: int) -> np.ndarray:
    """Running bin totals of genetoic: T[0] = bin, T[k+1] = T[k] + bin (double, in order).

    ``set_bins`` (LIB/gaboom.cpp:2295-2308) gives ``nbin = (max - min) / del``, rounded up,
    plus one for mapped (index) genes, and ``bin = 1 / nbin``. genetoic walks ``tot += bin``
    while ``tot < u``; the index it stops at is the first k with ``T[k] >= u``. The table is
    extended until it reaches 1.0 so that every u in [0, 1) lands inside it.
    """
    nbin = bin_count(gmin, gmax, gdel, gmap)
    b = 1.0 / nbin
    n = int(nbin) + 4
    t = np.cumsum(np.full(n, b, np.float64))   # numpy cumsum adds strictly left to right
    while t[-1] < 1.0:
        t = np.concatenate([t, t[-1] + np.cumsum(np.full(4, b))])
    return t


MAX_RANDOM_VALUE = 2147483647   # LIB/gaboom.h:36
RAND_MAX = 2147483647           # the C library's RAND_MAX on the reference's Linux builds


def random_double(gene: int) -> float:
    """RandomDouble(int32) (LIB/gaboom.cpp:2938-2940): a gene's place in [0, 1)."""
    return int(gene) / (float(MAX_RANDOM_VALUE) + 1.0)


def random_int(frac: float) -> int:
    """RandomInt (LIB/gaboom.cpp:2930-2935): frac scaled to [0, RAND_MAX], saturating."""
    raw = float(frac) * (float(RAND_MAX) + 1.0)
    if raw >= float(RAND_MAX) + 1.0:
        return RAND_MAX
    if raw < 0.0:
        return 0
    return int(raw)


def genetoic(tab: np.ndarray, gmin: float, gdel: float, gene: int) -> float:
    """genetoic (LIB/gaboom.cpp:2887-2906) of one gene with its running bin totals (gene_bins):
    min + del * (the first bin whose running total reaches RandomDouble(gene))."""
    i = int(np.searchsorted(tab, random_double(gene), side="left"))
    return float(gmin) + float(gdel) * float(i)


def ic_to_gene(gmin: float, gmax: float, gdel: float, gmap: int, ic: float) -> int:
    """ictogene (LIB/gaboom.cpp:2908-2927): the gene whose place is 1 - i * bin for the bin i
    of ic, as RandomInt gives it (used by the reference to seed chromosomes with given ICs)."""
    b = 1.0 / bin_count(gmin, gmax, gdel, gmap)
    i = int((float(ic) - float(gmin)) / float(gdel))
    tot = 1.0
    while i > 0:
        tot -= b
        i -= 1
    return random_int(tot)


def bin_count(gmin: float, gmax: float, gdel: float, gmap: int) -> float:
    """set_bins' nbin (LIB/gaboom.cpp:2295-2308): (max - min) / del, rounded up, one more for a
    mapped (index) gene."""
    nbin = (gmax - gmin) / gdel
    if nbin - int(nbin) > 0.0:
        nbin += 1.0
    if gmap:
        nbin += 1.0
    return nbin


def read_emat(path: str):
    """An energy-matrix file in the reference's format (read_emat, LIB/read_emat.cpp:8-148): the
    upper triangle of ntypes x ntypes, one line per type pair (i, j >= i) in order, the values
    after the "=" (or the whole line): one number is a single value (weight 1), an even count
    are the (x, y) points of a density curve (weight 0). ntypes follows from the line count.
    Returns (emat, emat_weight, emat_curves) as SystemInputs takes them."""
    with open(path) as f:
        lines = [ln for ln in f.read().split("\n")]
    if lines and lines[-1] == "":
        lines.pop()
    n = len(lines)
    t = int(round((-1.0 + (1.0 + 8.0 * n) ** 0.5) / 2.0))
    if t * (t + 1) // 2 != n:
        raise ValueError(f"{path}: {n} lines is not the upper triangle of a square matrix")
    emat = np.zeros((t, t), np.float32)
    weight = np.zeros((t, t), np.int32)
    curves = {}
    k = 0
    for i in range(t):
        for j in range(i, t):
            line = lines[k]
            k += 1
            if "=" in line:
                line = line[line.index("=") + 1:]
            vals = line.split()
            if len(vals) == 1:
                emat[i, j] = emat[j, i] = np.float32(float(vals[0]))
                weight[i, j] = weight[j, i] = 1
            elif vals and len(vals) % 2 == 0:
                pts = [(float(np.float32(float(vals[q]))), float(np.float32(float(vals[q + 1]))))
                       for q in range(0, len(vals), 2)]
                curves[(i, j)] = pts
            else:
                raise ValueError(f"{path}: line {k}: {len(vals)} values for pair {i + 1}-{j + 1}")
    return emat, weight, curves


def make_inputs(n_rec: int, cleft_radius: float, n_lig: int, n_tor: int, seed: int,
                spacing: float = 0.375, edge: float | None = None, side_chains: int = 0,
                rotamers: int = 8) -> SystemInputs:
    """One seeded docking system of the given shape (``edge``: receptor cube edge to start from;
    ``side_chains`` flexible residues of ``rotamers`` rotamers carved into the cleft wall)."""
    rec = synth.poisson_disc_receptor(n_rec, cleft_radius, seed=seed, edge=edge)
    if side_chains:
        rec = synth.add_flexible_residues(rec, side_chains, rotamers, seed=seed + 3)
    lig = synth.random_ligand(n_lig, n_tor, seed=seed + 1)
    grid = synth.cleft_grid(rec.cleft_center, cleft_radius, spacing)
    emat = synth.energy_matrix(seed + 2)
    return SystemInputs(receptor=rec, ligand=lig, grid_xyz=grid, emat=emat)
