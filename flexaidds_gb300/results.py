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
