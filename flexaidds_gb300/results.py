"""Result files of a docking run, written from the device results.

* ``cad_text`` / ``write_cad`` — the cluster table the reference writes after clustering
  (``<prefix>.cad``, LIB/cluster.cpp:184-216) from ``GPUEvaluator.cluster``'s result;
* ``par_bytes`` / ``write_par`` — the final population file ``<rrgfile>_par.res``
  (write_par, LIB/gaboom.cpp:2771-2803) from a population's int32 genes and the gene limits.

Formats are byte for byte the reference's: the .cad lines use its printf formats, and _par.res
is the 5-byte tag "genes", one genlim record per gene as the reference's struct lies in memory on
LP64 targets (max, min, del, bin, nbin as doubles, map as int32, 4 bytes of padding, written here
as zeros; LIB/gaboom.h:48-55), the 5-byte tag "chrom", then every chromosome's genes as int32.
"""
from __future__ import annotations

import struct

import numpy as np

from .system import Descriptor


def cad_text(res: dict) -> str:
    """The .cad file of a clustering result (LIB/cluster.cpp:184-216): one line per cluster
    formed, in the entries' final order, then the RMSD between every pair of cluster heads."""
    nc = int(res["n_clusters"])
    out = []
    for i in range(nc):
        out.append("Cluster %d: TOP=%d TCF=%f ACF=%f freq=%d\n" % (
            i, int(res["top"][i]), float(res["tcf"][i]), float(res["acf"][i]), int(res["freq"][i])))
    if nc > 1:
        out.append("RMSD between clusters\n")
        for i in range(nc):
            for j in range(i + 1, nc):
                out.append("rmsd(%d,%d)=%f\n" % (i, j, float(res["top_rmsd"][i][j])))
    return "".join(out)


def write_cad(prefix: str, res: dict) -> str:
    """Writes <prefix>.cad; returns its path."""
    path = prefix + ".cad"
    with open(path, "w") as f:
        f.write(cad_text(res))
    return path


def set_bins(gmin: float, gmax: float, gdel: float, gmap: int):
    """(bin, nbin) of one gene as set_bins computes them (LIB/gaboom.cpp:2291-2302)."""
    nbin = (gmax - gmin) / gdel
    if nbin - int(nbin) > 0.0:
        nbin += 1.0
    if gmap:
        nbin += 1.0
    return 1.0 / nbin, nbin


def par_bytes(desc: Descriptor, genes: np.ndarray) -> bytes:
    """Contents of the _par.res file for a population (P, n_genes) of int32 genes, in the order
    given (the reference writes its final population sorted by energy)."""
    genes = np.ascontiguousarray(genes, np.int32)
    if genes.ndim != 2 or genes.shape[1] != desc.n_genes:
        raise ValueError("genes must be (P, n_genes)")
    parts = [b"genes"]
    for g in range(desc.n_genes):
        gmin, gmax, gdel = float(desc.gene_min[g]), float(desc.gene_max[g]), float(desc.gene_del[g])
        gmap = int(desc.gene_map[g])
        b, nbin = set_bins(gmin, gmax, gdel, gmap)
        parts.append(struct.pack("<5di4x", gmax, gmin, gdel, b, nbin, gmap))
    parts.append(b"chrom")
    parts.append(genes.astype("<i4").tobytes())
    return b"".join(parts)


def write_par(path: str, desc: Descriptor, genes: np.ndarray) -> str:
    with open(path, "wb") as f:
        f.write(par_bytes(desc, genes))
    return path


def read_par(data: bytes, n_genes: int):
    """Parses _par.res contents: (gene limits as a list of (max, min, del, bin, nbin, map),
    genes (P, n_genes) int32)."""
    if data[:5] != b"genes":
        raise ValueError("not a _par.res file")
    off, lim = 5, []
    for _ in range(n_genes):
        lim.append(struct.unpack_from("<5di4x", data, off))
        off += 48
    if data[off:off + 5] != b"chrom":
        raise ValueError("not a _par.res file")
    off += 5
    genes = np.frombuffer(data[off:], dtype="<i4").reshape(-1, n_genes).astype(np.int32)
    return lim, genes


# ------------------------------------------------------------------------------------------
# Pose PDB files (write_pdb, LIB/write_pdb.cpp:91-170)
# ------------------------------------------------------------------------------------------

def element_of(atom_type: int) -> str:
    """The two-character element write_pdb prints for an atom type (get_element,
    LIB/write_pdb.cpp:218-300: the FlexAID type ranges of C, N, O and S, then one type per
    element; other types print blank)."""
    t = int(atom_type)
    for lo, hi, sym in ((1, 5, " C"), (6, 12, " N"), (13, 16, " O"), (17, 21, " S")):
        if lo <= t <= hi:
            return sym
    single = {22: " P", 23: " F", 24: "Cl", 25: "Br", 26: " I", 27: "Se", 28: "Mg", 29: "Sr", 30: "Cu",
              31: "Mn", 32: "Hg", 33: "Cd", 34: "Ni", 35: "Zn", 36: "Ca", 37: "Fe", 38: "Co", 39: "Du"}
    return single.get(t, "  ")


class PdbAtom:
    """One atom's record fields as the reference's atoms/residue arrays hold them: serial number,
    atom name (the PDB's four columns, spaces kept), residue name, chain, residue number,
    HETATM (ligand residue) or ATOM, FlexAID type."""
    __slots__ = ("number", "name", "resname", "chain", "resnum", "hetatm", "type")

    def __init__(self, number, name, resname, chain, resnum, hetatm, atom_type):
        self.number, self.name, self.resname = int(number), str(name), str(resname)
        self.chain, self.resnum, self.hetatm, self.type = str(chain), int(resnum), bool(hetatm), int(atom_type)


def pdb_atom_line(a: PdbAtom, xyz) -> str:
    """One coordinate record in write_pdb's format (LIB/write_pdb.cpp:130-141)."""
    return "%s%5d %s %s %c%4d    %8.3f%8.3f%8.3f  1.00  0.00          %2s  \n" % (
        "HETATM" if a.hetatm else "ATOM  ", a.number, a.name, a.resname, a.chain, a.resnum,
        float(xyz[0]), float(xyz[1]), float(xyz[2]), element_of(a.type))


def pose_pdb_text(remark: str, atoms, xyz, ligand_bonds=None, ligand_atoms=None) -> str:
    """A pose file laid out as write_pdb writes it: the generator line, the caller's remark
    block, one record per atom (receptor residues, with the rotamer each flexible side chain
    takes, then the ligand: coordinates in xyz, float32 as the reference keeps them), the CONECT
    records of the ligand atoms (ligand_atoms: their indices in atoms; ligand_bonds: per ligand
    atom the indices in atoms of its bonded atoms, in the order the reference stores them) and
    END. The reference's optional block of per-type contribution remarks (write_contributions)
    is not written."""
    out = ["REMARK coordinate file generated by FlexAID\n", remark + "\n"]
    xyz = np.asarray(xyz, np.float32)
    for k, a in enumerate(atoms):
        out.append(pdb_atom_line(a, xyz[k]))
    if ligand_atoms is not None:
        for k, j in enumerate(ligand_atoms):
            line = "CONECT%5d" % atoms[j].number
            for b in (ligand_bonds[k] if ligand_bonds is not None else []):
                line += "%5d" % atoms[b].number
            out.append(line + "\n")
    out.append("END\n")
    return "".join(out)
