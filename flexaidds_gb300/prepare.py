"""Set-up of a docking system: raw generator output -> ``Descriptor``.

Restates the reference's set-up steps that produce what the evaluation path reads:
  * receptor centre and bounds: calc_center (LIB/calc_center.cpp:8-61)
  * ligand internal coordinates: buildic (LIB/buildic.cpp:6-71) with the single-precision
    geometry of LIB/geometry.cpp (distance, bndang, dihedral)
  * rebuild order: buildlist for the whole ligand (LIB/buildlist.cpp:11-219, bnum = 0)
  * torsion shift cycles: assign_shift (LIB/assign_shift.cpp:9-116)
  * bonded matrix: bondedlist + update_bonded with bloops = 2 (LIB/bondedlist.cpp,
    LIB/update_bonded.cpp)
  * the first rebuild with buildcc and the ICs read back from it (LIB/read_lig.cpp:424-484,
    then buildic again inside add2_optimiz_vec)
  * cleft-grid ICs: calc_cleftic (LIB/calc_cleftic.cpp:5-33), entry 0 the initial anchor
  * genes: add2_optimiz_vec for the grid index, the three rotations and every flexible bond
    (LIB/add2_optimiz_vec.cpp:93-196) with the reference's default deltas (LIB/top.cpp:266-270),
    then one rotamer gene per flexible side chain (LIB/add2_optimiz_vec.cpp:28-60)
  * flexible side chains: the residue's bonded matrix (bondedlist + update_bonded, as
    build_rotamers makes it, LIB/build_rotamers.cpp:309-345); the rotamer coordinates are
    generator output here (the reference builds them from a rotamer library with buildcc)

The integer structure (rebuild order, cycles, bonded matrix, genes) is the reference's exactly;
the single-precision ICs agree to within a few units in the last place (transcendental
functions come from numpy here rather than the C library).
"""
from __future__ import annotations

import math

import numpy as np

from .system import Descriptor, SystemInputs

_PI = 3.141592          # LIB/flexaid.h:86
_F = np.float32


def calc_center(xyz: np.ndarray):
    """ori (float sequential mean), globalmin, globalmax, maxwidth of the receptor atoms."""
    xyz = np.asarray(xyz, np.float32)
    ori = np.empty(3, np.float32)
    for k in range(3):
        s = np.cumsum(xyz[:, k], dtype=np.float32)[-1]
        ori[k] = _F(s) / _F(xyz.shape[0])
    gmin = xyz.min(axis=0).astype(np.float32)
    gmax = xyz.max(axis=0).astype(np.float32)
    mw = _F(0.0)
    for k in range(3):
        d = _F(gmax[k] - gmin[k])
        if d > mw:
            mw = d
    return ori, gmin, gmax, float(mw)


def _frame(ori):
    ori = np.asarray(ori, np.float32)
    a = np.asarray([_F(1.0) + ori[0], _F(0.0) + ori[1], _F(0.0) + ori[2]], np.float32)
    b = np.asarray([_F(0.0) + ori[0], _F(0.0) + ori[1], _F(0.0) + ori[2]], np.float32)
    c = np.asarray([_F(0.0) + ori[0], _F(1.0) + ori[1], _F(0.0) + ori[2]], np.float32)
    return a, b, c


def _distance(a, b):
    d = (a - b).astype(np.float32)
    r2 = (d[..., 0] * d[..., 0]).astype(np.float32)
    r2 = (r2 + d[..., 1] * d[..., 1]).astype(np.float32)
    r2 = (r2 + d[..., 2] * d[..., 2]).astype(np.float32)
    return np.sqrt(r2).astype(np.float32)


def _bndang(a, b, c):
    u = (a - b).astype(np.float32)
    v = (c - b).astype(np.float32)
    cosa = np.zeros(np.broadcast(u[..., 0], v[..., 0]).shape, np.float32)
    absu = np.zeros_like(cosa)
    absv = np.zeros_like(cosa)
    for i in range(3):
        cosa = (cosa + u[..., i] * v[..., i]).astype(np.float32)
        absu = (absu + u[..., i] * u[..., i]).astype(np.float32)
        absv = (absv + v[..., i] * v[..., i]).astype(np.float32)
    cosa = (cosa / np.sqrt((absu * absv).astype(np.float32))).astype(np.float32)
    ang = np.arccos(cosa.astype(np.float64)).astype(np.float32)
    return (ang.astype(np.float64) * 180.0 / _PI).astype(np.float32)


def _cross(x2, x3):
    return np.stack([x2[..., 1] * x3[..., 2] - x3[..., 1] * x2[..., 2],
                     -x2[..., 0] * x3[..., 2] + x3[..., 0] * x2[..., 2],
                     x2[..., 0] * x3[..., 1] - x3[..., 0] * x2[..., 1]], axis=-1).astype(np.float32)


def _dot(a, b):
    s = (a[..., 0] * b[..., 0]).astype(np.float32)
    s = (s + a[..., 1] * b[..., 1]).astype(np.float32)
    return (s + a[..., 2] * b[..., 2]).astype(np.float32)


def _dihedral(a1, a2, a3, a4):
    r1 = (a2 - a1).astype(np.float32)
    r2 = (a3 - a2).astype(np.float32)
    r3 = (a4 - a3).astype(np.float32)
    n1 = _cross(r1, r2)
    n2 = _cross(r2, r3)
    psin = (_dot(n1, r3) * np.sqrt(_dot(r2, r2))).astype(np.float32)
    pcos = _dot(n1, n2)
    at = np.arctan2(psin.astype(np.float64), pcos.astype(np.float64)).astype(np.float32)
    return (_F(57.2958) * at).astype(np.float32)


def buildic(xyz, rec, ori):
    """dis/ang/dih of every ligand atom from its three references (-1 = frame point)."""
    fa, fb, fc = _frame(ori)
    n = xyz.shape[0]
    ic = np.zeros((n, 3), np.float32)
    for i in range(n):
        r0, r1, r2 = (int(v) for v in rec[i][:3])
        ca = xyz[r0] if r0 >= 0 else fa
        cb = xyz[r1] if r1 >= 0 else fb
        cc = xyz[r2] if r2 >= 0 else fc
        ci = xyz[i]
        ic[i, 0] = _distance(ci, ca)
        ic[i, 1] = _bndang(ci, ca, cb)
        ic[i, 2] = _dihedral(ci, ca, cb, cc)
    return ic


def buildcc(ic, rec, order, ori, xyz):
    """Cartesian coordinates from ICs along the rebuild order (LIB/buildcc.cpp:6-134)."""
    xyz = np.array(xyz, np.float32)
    ori = np.asarray(ori, np.float32)
    for l in order:
        X = np.zeros((4, 3), np.float32)
        for i in range(1, 4):
            j = int(rec[l][i - 1])
            if j >= 0:
                X[i] = xyz[j]
            elif i == 1:
                X[i] = [_F(1.0) + ori[0], _F(0.0) + ori[1], _F(0.0) + ori[2]]
            elif i == 3:
                X[i] = [_F(0.0) + ori[0], _F(1.0) + ori[1], _F(0.0) + ori[2]]
            else:
                X[i] = [_F(0.0) + ori[0], _F(0.0) + ori[1], _F(0.0) + ori[2]]
            X[i] = (X[i] + _F(1e-10)).astype(np.float32)
        x, y, z = X[:, 0], X[:, 1], X[:, 2]
        a = _F(_F(y[1] * _F(z[2] - z[3])) + _F(y[2] * _F(z[3] - z[1]))) + _F(y[3] * _F(z[1] - z[2]))
        b = _F(_F(z[1] * _F(x[2] - x[3])) + _F(z[2] * _F(x[3] - x[1]))) + _F(z[3] * _F(x[1] - x[2]))
        c = _F(_F(x[1] * _F(y[2] - y[3])) + _F(x[2] * _F(y[3] - y[1]))) + _F(x[3] * _F(y[1] - y[2]))
        op = _F(np.sqrt(_F(_F(a * a + b * b) + c * c)))
        cx, cy, cz = _F(a / op), _F(b / op), _F(c / op)
        a, b, c = _F(x[2] - x[1]), _F(y[2] - y[1]), _F(z[2] - z[1])
        d = _F(_F(1.0) / _F(np.sqrt(_F(_F(a * a + b * b) + c * c))))
        op = _F(ic[l][0] * d)
        xn, yn, zn = _F(a * op), _F(b * op), _F(c * op)
        a, b, c = _F(cx * cx), _F(cy * cy), _F(cz * cz)
        angPI = _F(float(ic[l][1]) * _PI / 180.0)
        ct, st = _F(math.cos(float(angPI))), _F(-math.sin(float(angPI)))
        op = _F(_F(1.0) - ct)
        xk = _F(_F(_F(_F(cx * cz * op) - cy * st) * zn) + _F(_F(_F(1.0) - a) * ct + a) * xn) + _F(_F(cx * cy * op) + cz * st) * yn
        yk = _F(_F(_F(_F(cy * cx * op) - cz * st) * xn) + _F(_F(_F(1.0) - b) * ct + b) * yn) + _F(_F(cy * cz * op) + cx * st) * zn
        zk = _F(_F(_F(_F(cz * cy * op) - cx * st) * yn) + _F(_F(_F(1.0) - c) * ct + c) * zn) + _F(_F(cz * cx * op) + cy * st) * xn
        dihPI = _F(float(ic[l][2]) * _PI / 180.0)
        ct, st = _F(math.cos(float(dihPI))), _F(math.sin(float(dihPI)))
        op = _F(_F(1.0) - ct)
        cx, cy, cz = _F(_F(x[2] - x[1]) * d), _F(_F(y[2] - y[1]) * d), _F(_F(z[2] - z[1]) * d)
        a, b, c = _F(cx * cx), _F(cy * cy), _F(cz * cz)
        xyz[l, 0] = _F(_F(_F(_F(_F(cx * cz * op) - cy * st) * zk) + _F(_F(_F(1.0) - a) * ct + a) * xk) + _F(_F(cx * cy * op) + cz * st) * yk) + x[1]
        xyz[l, 1] = _F(_F(_F(_F(_F(cy * cx * op) - cz * st) * xk) + _F(_F(_F(1.0) - b) * ct + b) * yk) + _F(_F(cy * cz * op) + cx * st) * zk) + y[1]
        xyz[l, 2] = _F(_F(_F(_F(_F(cz * cy * op) - cx * st) * yk) + _F(_F(_F(1.0) - c) * ct + c) * zk) + _F(_F(cz * cx * op) + cy * st) * xk) + z[1]
    return xyz


def buildlist(rec, gpa, n):
    """Whole-ligand rebuild order (LIB/buildlist.cpp, bnum = 0): GPA atoms first, then atoms
    whose three references are already placed, scanning the remaining list in passes."""
    lst = list(range(n))
    for j in range(3):
        i = lst.index(gpa[j])
        lst[i] = lst[j]
        lst[j] = gpa[j]
    out = lst[:3]
    rest = lst[3:]
    while rest:
        i = 0
        progressed = False
        while i < len(rest):
            refs = [int(r) for r in rec[rest[i]][:3]]
            if not any(r in rest for r in refs if r >= 0):
                out.append(rest.pop(i))
                progressed = True
                i += 1        # the reference's scan steps past the entry shifted into slot i
            else:
                i += 1
        if not progressed:
            raise ValueError("rebuild references form a cycle")
    return out


def assign_shift(rec, ic, bonds_adj, order, flex):
    """rec[3] cycles and shifts of the atoms sharing a flexible bond (LIB/assign_shift.cpp).
    Returns (rec3, shift, bond) where bond[j] is the atom that carries torsion j's gene."""
    n = len(order)
    rec3 = np.full(len(ic), -1, np.int32)
    shift = np.zeros(len(ic), np.float32)
    bond = [f[0] for f in flex]
    done = [False] * len(flex)
    for i in range(3, n):
        atom = order[i]
        shiftlist = [atom]
        hit = -1
        for j in range(len(flex)):
            if done[j]:
                continue
            if atom in flex[j][:3]:
                hit = j
                break
        if hit >= 0:
            parent = int(rec[atom][0])
            for nb in bonds_adj[parent]:
                if nb == atom:
                    continue
                for k in range(i + 1, n):
                    if order[k] == nb:
                        shiftlist.append(nb)
        if len(shiftlist) > 1:
            done[hit] = True
            bond[hit] = shiftlist[0]
            m = len(shiftlist)
            for j in range(m):
                k = (j + 1) % m
                rec3[shiftlist[j]] = shiftlist[k]
                shift[shiftlist[k]] = _F(ic[shiftlist[k]][2] - ic[shiftlist[j]][2])
    return rec3, shift, bond


def bonded_matrix(bonds_adj, n, loops=2):
    """residue.bonded: graph distance up to ``loops`` bonds, else -1."""
    m = np.full((n, n), -1, np.int8)
    for a in range(n):
        m[a, a] = 0
        frontier = [a]
        seen = {a}
        for depth in range(1, loops + 1):
            nxt = []
            for u in frontier:
                for v in bonds_adj[u]:
                    if v not in seen:
                        seen.add(v)
                        nxt.append(v)
                        m[a, v] = depth
            frontier = nxt
    return m


def cleft_ic(grid_xyz, ori):
    """calc_cleftic: dis/ang/dih of each grid point against the frame points around ori."""
    fa, fb, fc = _frame(ori)
    g = np.asarray(grid_xyz, np.float32)
    dis = _distance(g, fa)
    ang = _bndang(g, fa, fb)
    dih = _dihedral(g, np.broadcast_to(fa, g.shape), np.broadcast_to(fb, g.shape), np.broadcast_to(fc, g.shape))
    return np.stack([dis, ang, dih], axis=1).astype(np.float32)


_RECEPTOR_MEMO: list = []   # (receptor xyz, grid xyz, centre, cleft ICs) of recent receptors


def _receptor_setup(rec_xyz, grid_xyz):
    """calc_center and the cleft ICs of a receptor, remembered for the last few receptors (they
    depend on the receptor and its grid only, not on the ligand)."""
    for k, (x, g, c, ic) in enumerate(_RECEPTOR_MEMO):
        if x is rec_xyz and g is grid_xyz:
            return c, ic
    c = calc_center(rec_xyz)
    ic = cleft_ic(grid_xyz, c[0])
    _RECEPTOR_MEMO.insert(0, (rec_xyz, grid_xyz, c, ic))
    del _RECEPTOR_MEMO[8:]
    return c, ic


def prepare(inp: SystemInputs, receptor_setup=None) -> Descriptor:
    """The descriptor of one docking system. receptor_setup: ((ori, globalmin, globalmax,
    maxwidth), grid ICs) of the receptor and its grid when they are already known (the receptor
    cache of a server computes the grid and its ICs once, on the device); else calc_center and
    calc_cleftic here."""
    rec, lig = inp.receptor, inp.ligand
    if receptor_setup is None:
        receptor_setup = _receptor_setup(rec.xyz, inp.grid_xyz)
    (ori, gmin, gmax, mw), grid_ic = receptor_setup
    n = lig.xyz.shape[0]
    adj = [[] for _ in range(n)]
    for a, b in lig.bonds:
        adj[a].append(b)
        adj[b].append(a)
    lrec = np.asarray(lig.rec, np.int64)
    ic1 = buildic(lig.xyz, lrec, ori)
    order = buildlist(lrec, lig.gpa, n)
    rec3, shift, bond = assign_shift(lrec, ic1, adj, order, lig.flex)
    xyz2 = buildcc(ic1, lrec, order, ori, lig.xyz)
    ic2 = buildic(xyz2, lrec, ori)
    grid = np.zeros((inp.grid_xyz.shape[0] + 1, 3), np.float32)
    grid[0] = ic1[lig.gpa[0]]
    grid[1:] = grid_ic
    n_grid = grid.shape[0]
    # genes: grid index, three rotations, flexible bonds (LIB/add2_optimiz_vec.cpp)
    typ = [-1, 1, 2, 2] + [2] * len(lig.flex)
    atm = [lig.gpa[0], lig.gpa[1], lig.gpa[1], lig.gpa[2]] + list(bond)
    gmin_ = [1.0] + [-180.0] * (3 + len(lig.flex))
    gmax_ = [float(n_grid - 1)] + [180.0] * (3 + len(lig.flex))
    gdel = [1.0, 5.0, 5.0, 5.0] + [10.0] * len(lig.flex)
    gmap = [1, 0, 0, 0] + [0] * len(lig.flex)
    opt = [0.0, float(ic2[lig.gpa[1]][1]), float(ic2[lig.gpa[1]][2]), float(ic2[lig.gpa[2]][2])] + \
          [float(ic2[b][2]) for b in bond]
    # rotamer genes of the flexible side chains, last (add2_optimiz_vec "SC",
    # LIB/add2_optimiz_vec.cpp:28-60): 0 .. trot with the index delta, mapped
    flex = rec.flex
    for r, f in enumerate(flex):
        typ.append(4)
        atm.append(r)
        gmin_.append(0.0)
        gmax_.append(float(f.n_rot - 1))
        gdel.append(1.0)
        gmap.append(1)
        opt.append(0.0)
    fx = {}
    if flex:
        bonded = []
        for f in flex:
            adj_r = [[] for _ in range(f.natm)]
            for a, b in f.bonds:
                adj_r[a].append(b)
                adj_r[b].append(a)
            bonded.append(bonded_matrix(adj_r, f.natm).reshape(-1))
        fx = dict(flex_first=np.asarray([f.first for f in flex], np.int32),
                  flex_natm=np.asarray([f.natm for f in flex], np.int32),
                  flex_nrot=np.asarray([f.n_rot for f in flex], np.int32),
                  flex_isbb=np.concatenate([f.isbb for f in flex]).astype(np.int8),
                  flex_xyz=np.concatenate([f.rot_xyz.reshape(-1, 3) for f in flex]).astype(np.float32),
                  flex_bonded=np.concatenate(bonded).astype(np.int8),
                  flex_prob=np.asarray([f.prob for f in flex], np.float32))
    base = ic2.copy()
    lrec4 = np.concatenate([lrec.astype(np.int32), rec3[:, None]], axis=1)
    w, off, ex, ey = inp.emat_tables()
    return Descriptor(**fx,
        rec_xyz=rec.xyz.copy(), rec_radius=rec.radius.copy(), rec_type=rec.type.copy(), ori=ori,
        globalmin=gmin, globalmax=gmax, maxwidth=mw, grid_ic=grid, lig_radius=lig.radius.copy(),
        lig_type=lig.type.copy(), lig_rec=lrec4, lig_shift=shift, lig_ic=base,
        build_order=np.asarray(order, np.int32), bonded=bonded_matrix(adj, n),
        gene_typ=np.asarray(typ, np.int32), gene_atm=np.asarray(atm, np.int32),
        gene_min=np.asarray(gmin_, np.float64), gene_max=np.asarray(gmax_, np.float64),
        gene_del=np.asarray(gdel, np.float64), gene_map=np.asarray(gmap, np.int32),
        opt_par=np.asarray(opt, np.float64), ntypes=int(inp.emat.shape[0]), emat_weight=w,
        emat_off=off, emat_x=ex, emat_y=ey, permeability=inp.permeability,
        dee_clash=inp.dee_clash, intramolecular=inp.intramolecular, solventterm=inp.solventterm)
