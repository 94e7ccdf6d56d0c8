// fxe_flexaid_pack.cpp — the reference's set-up state as the C ABI's descriptors (host only: no
// CUDA call, so the packing can be checked without a device).
#include <cstring>

#include "fxe_flexaid.h"

namespace {

bool fail(std::string* err, const std::string& msg) {
    if (err) *err = msg;
    return false;
}

}  // namespace

bool fxe_flexaid_pack(const FA_Global* FA, const atom* atoms, const resid* residue, const gridpoint* cleftgrid,
                      FxeFlexaidPacked* out, std::string* err) {
    if (!FA || !atoms || !residue || !cleftgrid || !out) return fail(err, "null argument");
    FxeFlexaidPacked& P = *out;
    P = FxeFlexaidPacked();
    const resid* lig = FA->resligand;
    if (!lig) return fail(err, "no ligand residue");

    // receptor atoms in Calc order (index_protein, LIB/Vcontacts.cpp:1600-1625): residues in order,
    // atoms fatm[0] .. latm[0]; the ligand residue must come last, as its atoms follow the
    // receptor's in Calc
    P.calc_of_atom.assign((size_t)FA->atm_cnt + 2, -1);
    for (int r = 1; r <= FA->res_cnt; ++r) {
        const resid& res = residue[r];
        if (&res == lig) {
            if (r != FA->res_cnt) return fail(err, "the ligand residue is not the last residue");
            continue;
        }
        for (int a = res.fatm[0]; a <= res.latm[0]; ++a) {
            P.calc_of_atom[a] = (int32_t)P.rec_radius.size();
            for (int c = 0; c < 3; ++c) P.rec_xyz.push_back(atoms[a].coor[c]);
            P.rec_radius.push_back(atoms[a].radius);
            P.rec_type.push_back(atoms[a].type);
        }
    }
    const int n_rec = (int)P.rec_radius.size();
    // cleft grid ICs (calc_cleftic, LIB/calc_cleftic.cpp:5-33; entry 0 the initial anchor)
    for (int g = 0; g < FA->num_grd; ++g) {
        P.grid_ic.push_back(cleftgrid[g].dis);
        P.grid_ic.push_back(cleftgrid[g].ang);
        P.grid_ic.push_back(cleftgrid[g].dih);
    }
    // flexible side chains: every rotamer's copy of the residue's atoms (build_rotamers appends them,
    // fatm[rot] .. latm[rot]), backbone flags, bonded matrix, the chance of a rotamer move
    const int nflex = FA->nflxsc;
    if (nflex < 0 || nflex > 8) return fail(err, "more than 8 flexible side chains");
    P.flex.resize(nflex);
    P.flex_backbone.resize(nflex);
    P.flex_bonded.resize(nflex);
    P.flex_xyz.resize(nflex);
    for (int r = 0; r < nflex; ++r) {
        const resid& res = residue[FA->flex_res[r].inum];
        const int na = res.latm[0] - res.fatm[0] + 1, nr = res.trot + 1;
        const int first = P.calc_of_atom[res.fatm[0]];
        if (first < 0) return fail(err, "flexible side chain outside the receptor");
        for (int k = 0; k < na; ++k) P.flex_backbone[r].push_back((int8_t)(atoms[res.fatm[0] + k].isbb ? 1 : 0));
        for (int q = 0; q < nr; ++q)
            for (int k = 0; k < na; ++k)
                for (int c = 0; c < 3; ++c) P.flex_xyz[r].push_back(atoms[res.fatm[q] + k].coor[c]);
        for (int i = 0; i < na; ++i)
            for (int j = 0; j < na; ++j) P.flex_bonded[r].push_back((int8_t)res.bonded[i][j]);
        fxe_flex_residue& f = P.flex[r];
        f.first = first;
        f.n_atoms = na;
        f.n_rot = nr;
        f.prob = FA->flex_res[r].prob;
    }
    for (int r = 0; r < nflex; ++r) {   // pointers once the vectors stop growing
        P.flex[r].backbone = P.flex_backbone[r].data();
        P.flex[r].rot_xyz = P.flex_xyz[r].data();
        P.flex[r].bonded = P.flex_bonded[r].data();
    }

    // ligand: atoms fatm[0] .. latm[0] numbered from 0; the frame sentinel 0 becomes -1
    const int f0 = lig->fatm[0], n = lig->latm[0] - lig->fatm[0] + 1;
    if (n < 3 || n > 128) return fail(err, "ligand of fewer than 3 or more than 128 atoms");
    auto local = [&](int a, int* v) {
        if (a == 0) { *v = -1; return true; }
        if (a < f0 || a >= f0 + n) return false;
        *v = a - f0;
        return true;
    };
    for (int i = 0; i < n; ++i) {
        const atom& a = atoms[f0 + i];
        P.lig_radius.push_back(a.radius);
        P.lig_type.push_back(a.type);
        P.lig_shift.push_back(a.shift);
        P.lig_ic.push_back(a.dis);
        P.lig_ic.push_back(a.ang);
        P.lig_ic.push_back(a.dih);
        for (int j = 0; j < 4; ++j) {
            int v = -1;
            if (!local(a.rec[j], &v)) return fail(err, "a ligand atom is built from an atom outside the ligand");
            P.lig_rec.push_back(v);
        }
    }
    for (int i = 0; i < FA->nmov[0]; ++i) {
        int v = -1;
        if (!local(FA->mov[0][i], &v) || v < 0) return fail(err, "rebuild list names an atom outside the ligand");
        P.build_order.push_back(v);
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) P.bonded.push_back((int8_t)lig->bonded[i][j]);
    // genes (add2_optimiz_vec's map_par and the limits of ic_bounds)
    for (int g = 0; g < FA->npar; ++g) {
        const int t = FA->map_par[g].typ;
        int atm = -1;
        if (t == 4) {
            for (int r = 0; r < nflex; ++r)
                if (residue[FA->flex_res[r].inum].fatm[0] == FA->map_par[g].atm) atm = r;
            if (atm < 0) return fail(err, "rotamer gene names no flexible side chain");
        } else if (t == -1 || t == 0 || t == 1 || t == 2) {
            if (!local(FA->map_par[g].atm, &atm)) return fail(err, "gene names an atom outside the ligand");
        } else {
            return fail(err, "gene type " + std::to_string(t) + " (normal modes) is not evaluated on the device");
        }
        P.gene_type.push_back(t);
        P.gene_atom.push_back(atm);
        P.gene_min.push_back(FA->min_opt_par[g]);
        P.gene_max.push_back(FA->max_opt_par[g]);
        P.gene_del.push_back(FA->del_opt_par[g]);
        P.gene_map.push_back(FA->map_opt_par[g]);
    }
    // energy matrix: per ordered type pair its weight flag and curve points, in list order
    const int T = FA->ntypes;
    P.em_offset.push_back(0);
    for (int k = 0; k < T * T; ++k) {
        const energy_matrix& e = FA->energy_matrix[k];
        P.em_weight.push_back(e.weight);
        for (const energy_values* v = e.energy_values; v; v = v->next_value) {
            P.em_x.push_back(v->x);
            P.em_y.push_back(v->y);
        }
        P.em_offset.push_back((int32_t)P.em_x.size());
    }

    fxe_receptor_desc& R = P.receptor;
    R.n_atoms = n_rec;
    R.xyz = P.rec_xyz.data();
    R.radius = P.rec_radius.data();
    R.type = P.rec_type.data();
    for (int c = 0; c < 3; ++c) {
        R.ori[c] = FA->ori[c];
        R.globalmin[c] = FA->globalmin[c];
        R.globalmax[c] = FA->globalmax[c];
    }
    R.maxwidth = FA->maxwidth;
    R.n_grid = FA->num_grd;
    R.grid_ic = P.grid_ic.data();
    R.n_flex = nflex;
    R.flex = nflex ? P.flex.data() : nullptr;
    fxe_ligand_desc& L = P.ligand;
    L.n_atoms = n;
    L.radius = P.lig_radius.data();
    L.type = P.lig_type.data();
    L.rec = P.lig_rec.data();
    L.shift = P.lig_shift.data();
    L.ic = P.lig_ic.data();
    L.n_build = (int32_t)P.build_order.size();
    L.build_order = P.build_order.data();
    L.bonded = P.bonded.data();
    L.n_genes = FA->npar;
    L.gene_type = P.gene_type.data();
    L.gene_atom = P.gene_atom.data();
    L.gene_min = P.gene_min.data();
    L.gene_max = P.gene_max.data();
    L.gene_del = P.gene_del.data();
    L.gene_map = P.gene_map.data();
    P.emat.ntypes = T;
    P.emat.weight = P.em_weight.data();
    P.emat.offset = P.em_offset.data();
    P.emat.x = P.em_x.data();
    P.emat.y = P.em_y.data();
    P.params.permeability = FA->permeability;
    P.params.dee_clash = FA->dee_clash;
    P.params.intramolecular = FA->intramolecular;
    P.params.solventterm = FA->solventterm;
    return true;
}
