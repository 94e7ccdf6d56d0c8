"""Seeded synthetic docking inputs: receptors, ligands, cleft grids, energy matrices, genes.

The shapes follow the docking workloads this package is measured on:

* receptor: N heavy atoms placed by Poisson-disc sampling (minimum separation 2.8 A) in a cube
  of edge ``40 * (N / 2000) ** (1/3)`` A centred on the origin (2000 atoms at 2.8 A in a 40 A
  cube is close to the random-sequential-addition jamming limit, so larger receptors scale the
  cube to keep the density), with a spherical cleft carved out at the centre so the atom count
  is exact. Types are uniform over 1..40, radii come from the per-type table below.
* ligand: a seeded tree of heavy atoms with 1.53 A bonds and 109.5 degree angles, with a chosen
  number of rotatable torsions among the non-terminal tree edges.
* cleft grid: points of a 0.375 A lattice inside the cleft sphere.
* energy matrix: symmetric ``ntypes x ntypes`` with N(0, 1) entries in fp32, single-valued
  (area-weighted) entries.
* genes: uniform int32 in ``[0, 2**31 - 1]``.
* flexible side chains: receptor atoms at the cleft wall replaced by residues of four backbone
  atoms (N, CA, C, O) and a 4-6-atom branch (CB onwards) pointing into the cleft, with a set of
  rotamers that re-sample the branch's dihedrals; receptor atoms within reach of any rotamer are
  removed so that no rotamer clashes with the rigid atoms.

Nothing here reads the reference; everything is reproducible from the seed.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

NTYPES = 40

# Radii (A) per atom type, the SYBYL-derived table of LIB/assign_radii_types.cpp:19-146.
# Type 2 depends on the number of covalent bonds (1.72 A below three bonds, else 1.61 A).
# Type 40 (the solvent column of the energy matrix) has no entry in that table; 1.40 A (the
# probe radius) is used for it here.
_TYPE_RADIUS = {
    1: 1.88, 3: 1.88, 4: 1.76, 5: 1.88, 6: 1.64, 7: 1.64, 8: 1.64, 9: 1.64, 10: 1.64,
    11: 1.64, 12: 1.64, 13: 1.42, 14: 1.46, 15: 1.46, 16: 1.46, 17: 1.782, 18: 1.782,
    19: 1.782, 20: 1.782, 21: 1.782, 22: 1.871, 23: 1.560, 24: 1.735, 25: 1.978, 26: 2.094,
    27: 1.9, 28: 0.72, 29: 1.18, 30: 1.18, 31: 0.73, 32: 1.02, 33: 0.95, 34: 0.69, 35: 0.74,
    36: 1.00, 37: 0.61, 38: 0.65, 39: 2.0, 40: 1.40,
}


def type_radius(t: int, nbonds: int = 0) -> np.float32:
    if t == 2:
        return np.float32(1.72 if (3 - nbonds) > 0 else 1.61)
    return np.float32(_TYPE_RADIUS[int(t)])


# --------------------------------------------------------------------------------------------
# receptor
# --------------------------------------------------------------------------------------------

@dataclass
class Receptor:
    xyz: np.ndarray          # (N, 3) float32
    type: np.ndarray         # (N,) int32, 1..NTYPES
    radius: np.ndarray       # (N,) float32
    cleft_center: np.ndarray  # (3,) float32
    cleft_radius: float
    edge: float = 0.0         # cube edge used (A)
    flex: list = field(default_factory=list)   # FlexResidue, in Calc order


@dataclass
class FlexResidue:
    """A receptor residue with rotamers: its atoms are receptor atoms first .. first + natm - 1
    (Calc order N, CA, C, O, CB, ...); rotamer 0 is the conformation in the receptor arrays."""
    first: int
    isbb: np.ndarray          # (natm,) int8, 1 = backbone atom (not scored)
    rot_xyz: np.ndarray       # (n_rot, natm, 3) float32
    bonds: list               # residue-local (i, j)
    prob: float = 1.0         # GA: chance a child's rotamer gene mutates / an initial one is drawn

    @property
    def natm(self) -> int:
        return int(self.isbb.shape[0])

    @property
    def n_rot(self) -> int:
        return int(self.rot_xyz.shape[0])


def poisson_disc_receptor(n_atoms: int, cleft_radius: float, seed: int,
                          min_sep: float = 2.8, edge: float | None = None) -> Receptor:
    """Poisson-disc sample exactly ``n_atoms`` points in a cube, excluding a central sphere.

    The cube edge is ``40 * (n_atoms / 2000) ** (1/3)`` A unless given. Near the jamming
    density a larger cleft can leave too little room; the edge then grows in 1% steps until
    the maximal set holds ``n_atoms`` (the edge used is recorded on the result).
    """
    if edge is None:
        edge = 40.0 * (n_atoms / 2000.0) ** (1.0 / 3.0)
    for _ in range(40):
        try:
            return _poisson_disc(n_atoms, cleft_radius, seed, min_sep, edge)
        except ValueError:
            edge *= 1.01
    raise ValueError(f"could not place {n_atoms} atoms")


def _poisson_disc(n_atoms, cleft_radius, seed, min_sep, edge):
    """Bridson's sampling (k = 30 candidates in the shell [r, 2r] around a random active point),
    then up to 20,000 uniform darts. Candidates are tested against the placed points in blocks
    (a padded cell grid, cells of min_sep / sqrt(3), the 5^3 cells around each candidate) and
    against the candidates of their own block accepted before them, so that every candidate is
    accepted exactly when a one-at-a-time test would accept it."""
    rng = np.random.default_rng(seed)
    half = edge / 2.0
    r2min = min_sep * min_sep
    rc2 = cleft_radius * cleft_radius
    cell = min_sep / math.sqrt(3.0)
    ng = int(math.ceil(edge / cell))
    grid = -np.ones((ng + 4, ng + 4, ng + 4), dtype=np.int64)    # two cells of padding per side
    arr = np.zeros((n_atoms + 1, 3), np.float64)
    off = np.array([(a, b, c) for a in range(-2, 3) for b in range(-2, 3) for c in range(-2, 3)], np.int64)
    state = {"n": 0, "last": 0}

    def add_block(C):
        """Candidates C (k, 3) in order; returns the indices of the points placed."""
        kk = C.shape[0]
        inside = ~np.any(np.abs(C) > half, axis=1) & (np.einsum('ij,ij->i', C, C) >= rc2)
        placed = []
        if not inside.any():
            return placed
        G = np.clip(((C + half) / cell).astype(np.int64), 0, ng - 1)
        nb = G[:, None, :] + off[None, :, :] + 2
        idx = grid[nb[..., 0], nb[..., 1], nb[..., 2]]
        valid = idx >= 0
        d = arr[np.where(valid, idx, 0)] - C[:, None, :]
        d2 = np.einsum('ij,ij->i', d.reshape(-1, 3), d.reshape(-1, 3)).reshape(kk, -1)
        clear = ~np.any(valid & ~(d2 >= r2min), axis=1) & inside
        taken = []
        for i in np.nonzero(clear)[0]:
            if taken:
                e = C[taken] - C[i]
                if not np.all(np.einsum('ij,ij->i', e, e) >= r2min):
                    continue
            g = G[i]
            grid[g[0] + 2, g[1] + 2, g[2] + 2] = state["n"]
            arr[state["n"]] = C[i]
            placed.append(state["n"])
            state["n"] += 1
            taken.append(i)
            state["last"] = int(i)
            if state["n"] >= n_atoms:
                break
        return placed

    while True:
        if add_block(rng.uniform(-half, half, 3)[None]):
            break
    active = [0]
    k = 30
    while active and state["n"] < n_atoms:
        ai = int(rng.integers(len(active)))
        base = arr[active[ai]].copy()
        # candidates in the spherical shell [r, 2r]
        dirs = rng.normal(size=(k, 3))
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        radii = min_sep * (1.0 + rng.uniform(0.0, 1.0, k))
        placed = add_block(base + dirs * radii[:, None])
        if placed:
            active.extend(placed)
        else:
            active[ai] = active[-1]
            active.pop()
    # top up with random darts if the active list ran dry early: one uniform triple per try, up
    # to 20,000 tries; drawn in blocks, and when a block holds the dart that completes the set the
    # generator is rewound and only the darts used are drawn again
    tries = 0
    while state["n"] < n_atoms and tries < 20000:
        m = min(4096, 20000 - tries)
        saved = rng.bit_generator.state
        add_block(rng.uniform(-half, half, (m, 3)))
        if state["n"] >= n_atoms:
            used = state["last"] + 1
            rng.bit_generator.state = saved
            rng.uniform(-half, half, (used, 3))
            break
        tries += m
    if state["n"] < n_atoms:
        raise ValueError(f"cube of edge {edge:.1f} A holds only {state['n']} atoms at {min_sep} A")
    pts = arr
    xyz = np.asarray(pts[:n_atoms], dtype=np.float64).astype(np.float32)
    types = rng.integers(1, NTYPES + 1, size=n_atoms).astype(np.int32)
    radius = np.asarray([type_radius(t, 0) for t in types], dtype=np.float32)
    return Receptor(xyz=xyz, type=types, radius=radius,
                    cleft_center=np.zeros(3, np.float32), cleft_radius=float(cleft_radius),
                    edge=float(edge))


# --------------------------------------------------------------------------------------------
# ligand
# --------------------------------------------------------------------------------------------

@dataclass
class Ligand:
    xyz: np.ndarray            # (n, 3) float32, initial pose
    type: np.ndarray           # (n,) int32
    radius: np.ndarray         # (n,) float32
    bonds: list                # list of (i, j)
    parent: np.ndarray         # (n,) int32, -1 for the root
    rec: np.ndarray            # (n, 3) int32 reconstruction references, -1 = reference frame
    gpa: tuple                 # three global-positioning atoms
    flex: list = field(default_factory=list)  # per rotatable bond: atoms whose dihedral it sets


def _place(a, b, c, bond, ang_deg, dih_deg):
    """NeRF: position of d with |d-a| = bond, angle(d,a,b) = ang, dihedral(d,a,b,c) = dih."""
    ang = math.radians(ang_deg)
    dih = math.radians(dih_deg)
    bc = a - b
    bc /= np.linalg.norm(bc)
    n = np.cross(b - c, bc)
    n /= np.linalg.norm(n)
    m = np.cross(n, bc)
    d2 = np.array([-bond * math.cos(ang), bond * math.sin(ang) * math.cos(dih),
                   bond * math.sin(ang) * math.sin(dih)])
    return a + d2[0] * bc + d2[1] * m + d2[2] * n


def add_flexible_residues(rec: Receptor, n_res: int, n_rot: int, seed: int,
                          branch=(4, 6), clearance: float = 3.0) -> Receptor:
    """Receptor with ``n_res`` flexible residues of ``n_rot`` rotamers each (see module doc).

    Anchors are receptor atoms 0.5-3.5 A outside the cleft sphere, at least 9 A apart; each
    becomes the CA of a residue whose CB points at the cleft centre. Rigid atoms closer than
    ``clearance`` to an atom of any rotamer are removed."""
    rng = np.random.default_rng(seed)
    c = np.asarray(rec.cleft_center, np.float64)
    xyz = rec.xyz.astype(np.float64)
    dist = np.linalg.norm(xyz - c, axis=1)
    cand = np.flatnonzero((dist > rec.cleft_radius + 0.5) & (dist < rec.cleft_radius + 3.5))
    rng.shuffle(cand)
    anchors = []
    for k in cand:
        if all(np.linalg.norm(xyz[k] - xyz[a]) >= 9.0 for a in anchors):
            anchors.append(int(k))
        if len(anchors) == n_res:
            break
    if len(anchors) < n_res:
        raise ValueError(f"only {len(anchors)} anchors for {n_res} flexible residues")
    residues = {}
    for a in anchors:
        ca = xyz[a]
        u = (c - ca) / np.linalg.norm(c - ca)
        v = np.cross(u, [0.0, 0.0, 1.0] if abs(u[2]) < 0.9 else [1.0, 0.0, 0.0])
        v /= np.linalg.norm(v)
        w = np.cross(u, v)
        n_at = ca + 1.46 * (-0.34 * u + 0.94 * v)
        c_at = ca + 1.52 * (-0.34 * u - 0.47 * v + 0.82 * w)
        o_at = c_at + 1.23 * (-0.6 * u + 0.8 * w)
        cb = ca + 1.53 * u
        nb = int(rng.integers(branch[0], branch[1] + 1))    # CB and the atoms after it
        confs, chis = [], set()
        while len(confs) < n_rot:
            chi = tuple(int(rng.choice([-60, 60, 180])) for _ in range(nb - 1))
            if chi in chis and len(chis) < 3 ** (nb - 1):
                continue
            chis.add(chi)
            pts = [n_at, ca, c_at, o_at, cb]
            prev = (cb, ca, n_at)
            for x in chi:
                p = _place(prev[0], prev[1], prev[2], 1.53, 109.5, x + rng.normal(0.0, 8.0))
                pts.append(p)
                prev = (p, prev[0], prev[1])
            confs.append(np.asarray(pts))
        natm = 4 + nb
        types = rng.integers(1, NTYPES, size=natm).astype(np.int32)
        bonds = [(0, 1), (1, 2), (2, 3), (1, 4)] + [(4 + i, 5 + i) for i in range(nb - 1)]
        residues[a] = (np.asarray(confs, np.float32), types, bonds)
    # per-residue probabilities of the GA's rotamer moves, in the range of the reference's
    # internal per-residue-type values (0.05-0.55)
    probs = {a: float(np.float32(rng.uniform(0.05, 0.55))) for a in anchors}
    # rigid atoms within reach of any rotamer atom go (the anchors become the residues' CA)
    every = np.concatenate([r[0].reshape(-1, 3) for r in residues.values()]).astype(np.float64)
    keep = np.ones(len(xyz), bool)
    for k in range(len(xyz)):
        if k in residues:
            continue
        if np.min(np.linalg.norm(every - xyz[k], axis=1)) < clearance:
            keep[k] = False
    out_xyz, out_t, out_r, flex = [], [], [], []
    for k in range(len(xyz)):
        if k in residues:
            confs, types, bonds = residues[k]
            first = len(out_xyz)
            natm = confs.shape[1]
            flex.append(FlexResidue(first=first,
                                    isbb=np.asarray([1, 1, 1, 1] + [0] * (natm - 4), np.int8),
                                    rot_xyz=confs, bonds=bonds, prob=probs[k]))
            out_xyz.extend(confs[0])
            out_t.extend(types)
            out_r.extend(type_radius(t, 0) for t in types)
        elif keep[k]:
            out_xyz.append(rec.xyz[k])
            out_t.append(rec.type[k])
            out_r.append(rec.radius[k])
    return Receptor(xyz=np.asarray(out_xyz, np.float32), type=np.asarray(out_t, np.int32),
                    radius=np.asarray(out_r, np.float32), cleft_center=rec.cleft_center,
                    cleft_radius=rec.cleft_radius, edge=rec.edge, flex=flex)


def random_ligand(n_atoms: int, n_torsions: int, seed: int, bond: float = 1.53,
                  angle: float = 109.5, min_nonbonded: float = 2.6,
                  center=(0.0, 0.0, 0.0)) -> Ligand:
    """Seeded random tree ligand with ``n_torsions`` rotatable bonds.

    Atoms 0-1-2 form the global-positioning chain. Reconstruction references follow a
    Z-matrix: (parent, grandparent, great-grandparent), with atoms 0, 1, 2 standing in where
    the chain is too short, so that every atom moves rigidly with the positioning frame.
    A small tree may offer fewer non-terminal bonds than requested; it then gets them all.
    """
    if n_atoms < 4:
        raise ValueError("ligands need at least 4 atoms")
    rng = np.random.default_rng(seed)
    for _attempt in range(400):
        parent = np.full(n_atoms, -1, np.int64)
        deg = np.zeros(n_atoms, np.int64)
        parent[1] = 0
        parent[2] = 1
        deg[0] = 1
        deg[1] = 2
        deg[2] = 1
        okt = True
        for i in range(3, n_atoms):
            # drug-like shapes: at most three heavy neighbours, attachment biased towards
            # recently added atoms so that large ligands stay elongated rather than bushy
            cand = np.nonzero(deg[:i] < 3)[0]
            if cand.size == 0:
                okt = False
                break
            w = 0.6 ** (i - 1 - cand).astype(np.float64)
            p = int(rng.choice(cand, p=w / w.sum()))
            parent[i] = p
            deg[p] += 1
            deg[i] = 1
        if not okt:
            continue
        children = [[] for _ in range(n_atoms)]
        for i in range(1, n_atoms):
            children[parent[i]].append(i)
        # rotatable bonds (G, P): P a non-terminal child of G, excluding the 0-1 bond whose
        # torsion is a rigid-body gene.
        eligible = [(int(parent[p]), p) for p in range(2, n_atoms)
                    if children[p] and not (parent[p] == 0 and p == 1)]
        if len(eligible) < n_torsions and _attempt < 100:
            continue
        n_tor = min(n_torsions, len(eligible))
        # reconstruction references
        rec = np.full((n_atoms, 3), -1, np.int64)
        rec[1] = (0, -1, -1)
        rec[2] = (1, 0, -1)
        for x in range(3, n_atoms):
            p = parent[x]
            if p == 0:
                rec[x] = (0, 1, 2)
            elif parent[p] == 0:
                rec[x] = (1, 0, 2) if p == 1 else (p, 0, 1)
            else:
                g = parent[p]
                rec[x] = (p, g, parent[g])
        # coordinates: BFS order guarantees references are placed first
        order = [0]
        head = 0
        while head < len(order):
            for c in children[order[head]]:
                order.append(c)
            head += 1
        adj = [set() for _ in range(n_atoms)]
        for i in range(1, n_atoms):
            adj[i].add(int(parent[i]))
            adj[int(parent[i])].add(i)
        near = [set([i]) | adj[i] | set().union(*[adj[j] for j in adj[i]]) for i in range(n_atoms)]
        placed_ok = False
        for _geo in range(8):
            xyz = np.zeros((n_atoms, 3))
            xyz[0] = center
            xyz[1] = xyz[0] + np.array([bond, 0.0, 0.0])
            th = math.radians(angle)
            xyz[2] = xyz[1] + bond * np.array([-math.cos(th), math.sin(th), 0.0])
            placed = [0, 1, 2]
            failed = False
            # place the children of each parent together, retrying the sibling base dihedral
            # until none of them comes closer than min_nonbonded to an already placed atom
            for p in order:
                kids = [x for x in children[p] if x >= 3]
                if not kids:
                    continue
                good = None
                for _try in range(16):
                    if p == 0:
                        dset = [60.0, 180.0, 300.0]
                    elif p == 1:
                        dset = [120.0, 240.0]
                    else:
                        b0 = float(rng.choice([60.0, 180.0, 300.0])) + float(rng.uniform(-30, 30))
                        dset = [b0, b0 + 120.0, b0 + 240.0]
                    pos = []
                    for s, x in enumerate(kids):
                        r0, r1, r2 = rec[x]
                        dih = dset[s % len(dset)] + float(rng.uniform(-8.0, 8.0))
                        pos.append(_place(xyz[r0], xyz[r1], xyz[r2], bond, angle, dih))
                    clash = False
                    for s, x in enumerate(kids):
                        others = [q for q in placed if q not in near[x]]
                        others += [kids[t] for t in range(s) if kids[t] not in near[x]]
                        if others:
                            q = np.asarray([xyz[o] if o in placed else pos[kids.index(o)] for o in others])
                            if np.min(np.linalg.norm(q - pos[s], axis=1)) < min_nonbonded:
                                clash = True
                                break
                    if not clash:
                        good = pos
                        break
                if good is None:
                    failed = True
                    break
                for s, x in enumerate(kids):
                    xyz[x] = good[s]
                    placed.append(x)
            if not failed:
                placed_ok = True
                break
        if not placed_ok:
            continue
        pick = rng.choice(len(eligible), size=n_tor, replace=False) if n_tor else []
        flex = []
        for k in sorted(int(i) for i in pick):
            g, p = eligible[k]
            flex.append(sorted(children[p])[:3])
        bonds = [(int(parent[i]), i) for i in range(1, n_atoms)]
        nb = np.bincount(np.asarray([b for e in bonds for b in e]), minlength=n_atoms)
        types = rng.integers(1, NTYPES + 1, size=n_atoms).astype(np.int32)
        radius = np.asarray([type_radius(t, int(nb[i])) for i, t in enumerate(types)], np.float32)
        return Ligand(xyz=xyz.astype(np.float32), type=types, radius=radius, bonds=bonds,
                      parent=parent.astype(np.int32), rec=rec.astype(np.int32), gpa=(0, 1, 2),
                      flex=flex)
    raise RuntimeError("could not generate a ligand with the requested torsions")


# --------------------------------------------------------------------------------------------
# cleft grid, energy matrix, genes
# --------------------------------------------------------------------------------------------

def cleft_grid(center, radius: float, spacing: float = 0.375) -> np.ndarray:
    """Lattice points strictly inside one cleft sphere, in the reference's scan order.

    Follows LIB/generate_grid.cpp:32-95 for a single sphere: the lattice starts at
    ``(int)((c - r) / s) * s`` per axis and runs while below ``((int)((c + r) / s) + 1) * s``,
    x fastest, keeping points with float squared distance below ``r * r``.
    """
    s = np.float32(spacing)
    c = np.asarray(center, np.float32)
    r = np.float32(radius)
    inv = np.float32(1.0) / s
    if float(inv - np.float32(int(inv))) <= 0.001:
        raise NotImplementedError("integer 1/spacing lattices are not generated here")
    lo = np.asarray([np.float32(int((float(c[k]) - float(r)) / float(s))) * s for k in range(3)], np.float32)
    hi = np.asarray([np.float32(int((float(c[k]) + float(r)) / float(s)) + 1.0) * s for k in range(3)], np.float32)
    axes = []
    for k in range(3):
        vals = []
        v = lo[k]
        while v < hi[k]:
            vals.append(v)
            v = np.float32(v + s)
        axes.append(np.asarray(vals, np.float32))
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing='ij')
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.float32)
    d = pts - c
    d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]).astype(np.float32)
    d2 = (d2 + d[:, 2] * d[:, 2]).astype(np.float32)
    keep = d2 < np.float32(r * r)
    return pts[keep]


def energy_matrix(seed: int, ntypes: int = NTYPES) -> np.ndarray:
    """Symmetric ntypes x ntypes matrix of N(0, 1) fp32 single values."""
    rng = np.random.default_rng(seed)
    m = rng.normal(size=(ntypes, ntypes)).astype(np.float32)
    return np.triu(m) + np.triu(m, 1).T


def random_genes(n_chrom: int, n_genes: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2 ** 31, size=(n_chrom, n_genes), dtype=np.int64).astype(np.int32)


def clustered_ensemble(desc, n_centres: int, per_centre: int, seed: int, spread: int = 2):
    """A seeded stand-in for a GA ensemble with structure to cluster: n_centres chromosomes drawn
    at random, each with per_centre variants whose genes move a few bins from the centre's
    (the grid index by up to 3 * spread points, each angle by up to spread bins), the values
    kept on their bins (min + del * i, as genetoic gives them) and within the gene limits.
    Energies are drawn around a per-centre mean; the rows come sorted by energy, best first.
    Returns (ic (n, n_genes), app_evalue (n,))."""
    rng = np.random.default_rng(seed)
    ng = desc.n_genes
    base = desc.genes_to_ic(random_genes(n_centres, ng, seed + 1))
    lo = np.zeros(ng, np.int64)
    hi = np.floor((desc.gene_max - desc.gene_min) / desc.gene_del + 1e-9).astype(np.int64)
    idx = np.rint((base - desc.gene_min) / desc.gene_del).astype(np.int64)           # (C, ng)
    mean = rng.normal(-25.0, 6.0, size=n_centres)
    step = rng.integers(-spread, spread + 1, size=(n_centres, per_centre, ng))
    step[:, :, desc.gene_typ == -1] *= 3
    step[:, :, desc.gene_typ == 4] = 0
    k = np.clip(idx[:, None, :] + step, lo, hi).reshape(-1, ng)
    ic = desc.gene_min + desc.gene_del * k.astype(np.float64)
    e = (mean[:, None] + rng.normal(0.0, 1.5, size=(n_centres, per_centre))).reshape(-1)
    order = np.argsort(e, kind="stable")
    return np.ascontiguousarray(ic[order]), np.ascontiguousarray(e[order])
