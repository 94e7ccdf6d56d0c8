// ref_harness.cpp — drives the reference FlexAID∆S scoring chain on synthetic inputs.
//
// TEST INFRASTRUCTURE ONLY. This file is compiled together with the reference's own sources
// (LIB/*.cpp, read in place from the reference checkout by oracle/Makefile) into
// oracle/_ref/libfxe_ref.so. Only tests/, the smoke check and the bench's CPU-baseline leg
// use it, and only as the checker.
//
// It replaces the reference's file readers (read_input / read_lig / read_pdb) by filling the
// FA/atoms/residue structures in memory, then runs the reference's own set-up functions in
// the order the reference runs them:
//   * defaults and VC allocation: LIB/top.cpp:200-345 and LIB/top.cpp:1011-1043
//   * receptor centre and bounds: calc_center (LIB/calc_center.cpp:8-61)
//   * ligand ICs, rebuild list, torsion shift cycles, bonded matrix, first rebuild:
//     LIB/read_lig.cpp:424-484 (buildic, buildlist, assign_shift, bondedlist/update_bonded,
//     buildcc)
//   * cleft grid ICs and bounds: LIB/generate_grid.cpp:26-30, calc_cleftic, ic_bounds
//   * genes: add2_optimiz_vec for translation, rotation and every flexible bond
//     (LIB/top.cpp:968-985 order), update_optres, create_rebuild_list (LIB/top.cpp:1119)
//   * first ic2cf with VC->recalc = 1, then VC->recalc = 0 (LIB/top.cpp:1132-1133)
// and evaluates chromosomes through eval_chromosome semantics (LIB/gaboom.cpp:1845-1866:
// clamp each IC into its gene limits, then ic2cf).

#include "flexaid.h"
#include "gaboom.h"
#include "Vcontacts.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <array>
#include <cstring>
#include <utility>
#include <vector>

extern "C" {

struct ref_input {
    int32_t n_rec;
    const float* rec_xyz;
    const int32_t* rec_type;
    const float* rec_radius;
    int32_t n_lig;
    const float* lig_xyz;
    const int32_t* lig_type;
    const float* lig_radius;
    int32_t n_bonds;
    const int32_t* bonds;       // n_bonds * 2, ligand-local
    const int32_t* lig_rec;     // n_lig * 3, ligand-local, -1 = reference frame
    int32_t gpa[3];
    int32_t n_flex;
    const int32_t* flex;        // n_flex * 3, ligand-local, -1 = unused slot
    int32_t n_grid;             // cleft points, not counting entry 0
    const float* grid_xyz;
    int32_t ntypes;
    const int32_t* emat_weight; // ntypes*ntypes (1 = single value, 0 = density curve)
    const int32_t* emat_off;    // ntypes*ntypes + 1 offsets into curve arrays
    const float* emat_x;
    const float* emat_y;
    float permeability;
    float dee_clash;
    int32_t intramolecular;
    float solventterm;
    // flexible side chains: residues of receptor atoms first .. first + natm - 1 (receptor-local,
    // ascending), with rotamer coordinates (rotamer 0 = the receptor's) and intra-residue bonds
    int32_t n_flexres;
    const int32_t* flex_first;
    const int32_t* flex_natm;
    const int32_t* flex_nrot;
    const int8_t* flex_isbb;    // concatenated per residue
    const float* flex_xyz;      // concatenated per residue: nrot * natm * 3
    const int32_t* flex_nbonds;
    const int32_t* flex_bonds;  // concatenated per residue: nbonds * 2, residue-local
};

struct ref_export_sizes {
    int32_t n_atoms;     // Calc atoms (receptor + ligand)
    int32_t n_lig;
    int32_t n_genes;
    int32_t n_grid;      // including entry 0
    int32_t n_mov;
};

}  // extern "C"

namespace {

struct Harness {
    FA_Global* FA = nullptr;
    VC_Global* VC = nullptr;
    atom* atoms = nullptr;
    resid* residue = nullptr;
    gridpoint* cleftgrid = nullptr;
    int n_rec = 0, n_lig = 0, lig_res = 0;
    std::vector<int> sc_slot;   // Calc indices of the scored side-chain atoms
    // every side-chain atom of every rotamer (atoms[] index, coordinates as given), so that the
    // coordinates can be put back before each pose (see ref_eval)
    std::vector<std::pair<int, std::array<float, 3>>> rotamer_atoms;
    std::vector<std::vector<int>> last_contacts;  // per ligand atom: partner Calc indices
    std::vector<std::vector<double>> last_areas;
    std::vector<std::vector<double>> last_dists;
};

Harness* H = nullptr;

int to_internal(const Harness& h, int local) { return local < 0 ? 0 : h.n_rec + 1 + local; }
int to_local(const Harness& h, int internal) { return internal == 0 ? -1 : internal - h.n_rec - 1; }

void set_defaults(FA_Global* FA, VC_Global* VC) {
    // LIB/top.cpp:200-345 (the fields the scoring chain reads)
    FA->contacts = (int*)calloc(MAX_ATOM_NUMBER, sizeof(int));
    VC->ptorder = (ptindex*)malloc(MAX_PT * sizeof(ptindex));
    VC->centerpt = (vertex*)malloc(MAX_PT * sizeof(vertex));
    VC->poly = (vertex*)malloc(MAX_POLY * sizeof(vertex));
    VC->cont = (plane*)malloc(MAX_PT * sizeof(plane));
    VC->vedge = (edgevector*)malloc(MAX_POLY * sizeof(edgevector));
    VC->recalc = 1;
    FA->MIN_NUM_ATOM = 1000;
    FA->MIN_NUM_RESIDUE = 250;
    FA->MIN_ROTAMER_LIBRARY_SIZE = 155;
    FA->MIN_ROTAMER = 1;
    FA->MIN_FLEX_BONDS = 5;
    FA->MIN_CLEFTGRID_POINTS = 250;
    FA->MIN_PAR = 6;
    FA->MIN_FLEX_RESIDUE = 5;
    FA->MIN_NORMAL_GRID_POINTS = 250;
    FA->MIN_OPTRES = 1;
    FA->MIN_CONSTRAINTS = 1;
    FA->vindex = 0;
    FA->dee_clash = 0.5;
    FA->intrafraction = 1.0;
    FA->rotamer_permeability = 0.8;
    FA->interaction_factor = 5.0;
    FA->htpmode = true;          // silences the rebuild-list prints
    FA->delta_angstron = 0.25;
    FA->delta_angle = 5.0;
    FA->delta_dihedral = 5.0;
    FA->delta_flexible = 10.0;
    FA->delta_index = 1.0;
    FA->deelig_flex = 0;
    FA->useacs = 0;
    FA->acsweight = 1.0;
    FA->remove_water = 1;
    FA->normalize_area = 0;
    FA->spacer_length = 0.375;
    FA->pbloops = 1;
    FA->bloops = 2;
    FA->permeability = 1.0;
    FA->intramolecular = 1;
    FA->solventterm = 0.0f;
    FA->dielectric = 4.0f;
    FA->useflexdee = 0;
    FA->omit_buried = 0;
    FA->vcontacts_planedef = 'X';
    strcpy(FA->vcontacts_self_consistency, "MAX");
    strcpy(FA->complf, "VCT");
    strcpy(FA->rngopt, "locclf");
    FA->num_atm = (int*)calloc(MAX_ATOM_NUMBER, sizeof(int));
    FA->map_par = (optmap*)calloc(FA->MIN_PAR, sizeof(optmap));
    FA->opt_par = (double*)calloc(FA->MIN_PAR, sizeof(double));
    FA->del_opt_par = (double*)calloc(FA->MIN_PAR, sizeof(double));
    FA->min_opt_par = (double*)calloc(FA->MIN_PAR, sizeof(double));
    FA->max_opt_par = (double*)calloc(FA->MIN_PAR, sizeof(double));
    FA->map_opt_par = (int*)calloc(FA->MIN_PAR, sizeof(int));
    FA->map_par_flexbond_first_index = -1;
    FA->map_par_sidechain_first_index = -1;
}

void free_harness(Harness* h) {
    if (!h) return;
    // The reference structures are process-lifetime allocations in the reference program;
    // the harness leaks them deliberately rather than guessing the reference's ownership.
    delete h;
}

}  // namespace

extern "C" {

int ref_setup(const ref_input* in) {
    free_harness(H);
    H = new Harness();
    Harness& h = *H;
    h.FA = new FA_Global();
    h.VC = new VC_Global();
    FA_Global* FA = h.FA;
    VC_Global* VC = h.VC;
    set_defaults(FA, VC);
    FA->permeability = in->permeability;
    FA->dee_clash = in->dee_clash;
    FA->intramolecular = in->intramolecular;
    FA->solventterm = in->solventterm;

    h.n_rec = in->n_rec;
    h.n_lig = in->n_lig;
    const int N = in->n_rec, n = in->n_lig;
    int n_copies = 0;
    for (int r = 0; r < in->n_flexres; ++r) n_copies += (in->flex_nrot[r] - 1) * in->flex_natm[r];
    const int natoms_alloc = N + n + n_copies + 2;
    h.atoms = (atom*)calloc(natoms_alloc, sizeof(atom));
    h.residue = (resid*)calloc(N + 3, sizeof(resid));
    atom* atoms = h.atoms;
    resid* residue = h.residue;

    // receptor: one residue per atom (protein type), except the flexible side chains, whose
    // atoms form one residue each (backbone flags, intra-residue bonds)
    std::vector<int> flex_res(in->n_flexres, 0), isbb_off(in->n_flexres, 0), xyz_off(in->n_flexres, 0),
        bond_off(in->n_flexres, 0);
    for (int r = 1; r < in->n_flexres; ++r) {
        isbb_off[r] = isbb_off[r - 1] + in->flex_natm[r - 1];
        xyz_off[r] = xyz_off[r - 1] + in->flex_nrot[r - 1] * in->flex_natm[r - 1] * 3;
        bond_off[r] = bond_off[r - 1] + in->flex_nbonds[r - 1] * 2;
    }
    int nres = 0, fr = 0;
    for (int k = 1; k <= N; ++k) {
        atom& a = atoms[k];
        for (int j = 0; j < 3; ++j) a.coor[j] = a.coor_ori[j] = in->rec_xyz[(k - 1) * 3 + j];
        a.number = k;
        a.radius = in->rec_radius[k - 1];
        a.type = in->rec_type[k - 1];
        a.recs = 'r';
        a.acs = -1.0f;
        FA->num_atm[k] = k;
        const bool starts = fr < in->n_flexres && in->flex_first[fr] == k - 1;
        const bool inside = fr > 0 && k - 1 < in->flex_first[fr - 1] + in->flex_natm[fr - 1];
        if (inside) {
            a.ofres = nres;
            a.isbb = in->flex_isbb[isbb_off[fr - 1] + (k - 1 - in->flex_first[fr - 1])];
            continue;
        }
        resid& r = residue[++nres];
        a.ofres = nres;
        r.type = 0;
        r.number = nres;
        r.chn = 'A';
        strcpy(r.name, "REC");
        if (starts) {
            const int nr = in->flex_nrot[fr], na = in->flex_natm[fr];
            r.fatm = (int*)calloc(nr, sizeof(int));
            r.latm = (int*)calloc(nr, sizeof(int));
            r.fatm[0] = k;
            r.latm[0] = k + na - 1;
            strcpy(r.name, "FLX");
            a.isbb = in->flex_isbb[isbb_off[fr]];
            flex_res[fr] = nres;
            ++fr;
        } else {
            r.fatm = (int*)malloc(sizeof(int));
            r.latm = (int*)malloc(sizeof(int));
            r.fatm[0] = r.latm[0] = k;
        }
    }
    for (int r = 0; r < in->n_flexres; ++r)
        for (int b = 0; b < in->flex_nbonds[r]; ++b) {
            const int x = in->flex_first[r] + 1 + in->flex_bonds[bond_off[r] + 2 * b];
            const int y = in->flex_first[r] + 1 + in->flex_bonds[bond_off[r] + 2 * b + 1];
            atoms[x].bond[++atoms[x].bond[0]] = y;
            atoms[y].bond[++atoms[y].bond[0]] = x;
        }
    FA->res_cnt = nres;
    FA->atm_cnt = N;
    FA->atm_cnt_real = N;
    calc_center(FA, atoms, residue);

    // ligand residue
    const int L = nres + 1;
    h.lig_res = L;
    FA->res_cnt = L;
    resid& lr = residue[L];
    lr.fatm = (int*)malloc(sizeof(int));
    lr.latm = (int*)malloc(sizeof(int));
    lr.fatm[0] = N + 1;
    lr.latm[0] = N + n;
    lr.bond = (int*)calloc(in->n_flex + 6, sizeof(int));
    lr.gpa = (int*)malloc(3 * sizeof(int));
    lr.type = 1;
    lr.number = 1;
    lr.chn = ' ';
    lr.rot = 0;
    lr.fdih = in->n_flex;
    strcpy(lr.name, "LIG");
    FA->resligand = &residue[L];
    for (int i = 0; i < n; ++i) {
        atom& a = atoms[N + 1 + i];
        for (int j = 0; j < 3; ++j) a.coor[j] = a.coor_ori[j] = in->lig_xyz[i * 3 + j];
        a.number = 90001 + i;
        FA->num_atm[a.number] = N + 1 + i;
        a.radius = in->lig_radius[i];
        a.type = in->lig_type[i];
        a.ofres = L;
        a.recs = 'm';
        a.acs = -1.0f;
        for (int j = 0; j < 3; ++j) a.rec[j] = to_internal(h, in->lig_rec[i * 3 + j]);
        a.rec[3] = 0;
    }
    for (int b = 0; b < in->n_bonds; ++b) {
        int x = N + 1 + in->bonds[2 * b], y = N + 1 + in->bonds[2 * b + 1];
        atoms[x].bond[++atoms[x].bond[0]] = y;
        atoms[y].bond[++atoms[y].bond[0]] = x;
    }
    for (int j = 0; j < 3; ++j) lr.gpa[j] = N + 1 + in->gpa[j];
    FA->atm_cnt = N + n;
    FA->atm_cnt_real = N + n;     // rotamer copies added below do not join Calc
    FA->num_het = 1;
    FA->num_het_atm = n;

    // LIB/read_lig.cpp:424-484 (ICs from the generated coordinates instead of an .ic file)
    buildic(FA, atoms, residue, L);
    int natm = 0;
    std::vector<int> list(n + 4, 0);
    buildlist(FA, atoms, residue, L, 0, &natm, list.data());
    std::vector<int*> altfdih(in->n_flex + 1, nullptr);
    std::vector<int> altstore((in->n_flex + 1) * 3, 0);
    for (int j = 1; j <= in->n_flex; ++j) {
        altfdih[j] = &altstore[j * 3];
        for (int k = 0; k < 3; ++k) {
            int loc = in->flex[(j - 1) * 3 + k];
            altfdih[j][k] = loc < 0 ? 0 : N + 1 + loc;
            if (lr.bond[j] == 0 && altfdih[j][k] != 0) lr.bond[j] = altfdih[j][k];
        }
    }
    altfdih[0] = &altstore[0];
    if (lr.fdih > 0) assign_shift(atoms, residue, L, natm, list.data(), altfdih.data());
    FA->optres = (OptRes*)calloc(2, sizeof(OptRes));
    FA->optres[0].rnum = L;
    FA->optres[0].type = 1;
    FA->optres[0].tot = n;
    FA->num_optres = 1;
    {
        std::vector<int> bondlist(MAX_ATM_HET), neighbours(MAX_ATM_HET);
        for (int i = 0; i < natm; ++i) {
            int nbonded = 0;
            bondedlist(atoms, list[i], FA->bloops, &nbonded, bondlist.data(), neighbours.data());
            update_bonded(&residue[L], natm, nbonded, bondlist.data(), neighbours.data());
        }
    }
    buildcc(FA, atoms, natm, list.data());
    for (int i = N + 1; i <= N + n; ++i)
        for (int j = 0; j < 3; ++j) atoms[i].coor_ori[j] = atoms[i].coor[j];

    // flexible side chains as build_rotamers leaves them (LIB/build_rotamers.cpp:84-135,
    // 300-350): each rotamer a copy of the residue's atoms appended after the last atom, with the
    // rotamer's coordinates (given here instead of built from a rotamer library); an optimised
    // residue of type 0 with its bonded matrix; the residue listed in FA->flex_res
    FA->atm_cnt = N + n;
    if (in->n_flexres > 0) {
        FA->optres = (OptRes*)realloc(FA->optres, (size_t)(1 + in->n_flexres) * sizeof(OptRes));
        memset(&FA->optres[1], 0, (size_t)in->n_flexres * sizeof(OptRes));
        FA->flex_res = (flxsc*)calloc(in->n_flexres, sizeof(flxsc));
        std::vector<int> bondlist(MAX_ATM_HET), neighbours(MAX_ATM_HET);
        for (int r = 0; r < in->n_flexres; ++r) {
            const int kres = flex_res[r], na = in->flex_natm[r], nr = in->flex_nrot[r];
            resid& res = residue[kres];
            for (int rot = 1; rot < nr; ++rot) {
                const int delta = FA->atm_cnt - res.fatm[0] + 1;
                res.fatm[rot] = res.fatm[0] + delta;
                res.latm[rot] = res.latm[0] + delta;
                for (int j = res.fatm[0]; j <= res.latm[0]; ++j) {
                    atoms[j + delta] = atoms[j];
                    for (int c = 0; c < 3; ++c)
                        atoms[j + delta].coor[c] = atoms[j + delta].coor_ori[c] =
                            in->flex_xyz[xyz_off[r] + ((rot * na) + (j - res.fatm[0])) * 3 + c];
                }
                FA->atm_cnt += na;
            }
            for (int rot = 0; rot < nr; ++rot)
                for (int k = 0; k < na; ++k) {
                    const int a = res.fatm[rot] + k;
                    h.rotamer_atoms.push_back({a, {atoms[a].coor[0], atoms[a].coor[1], atoms[a].coor[2]}});
                }
            res.trot = nr - 1;
            res.rot = 0;
            FA->optres[1 + r].rnum = kres;
            FA->optres[1 + r].type = 0;
            FA->optres[1 + r].tot = na;
            for (int i = 0; i < na; ++i) {
                int nbonded = 0;
                bondedlist(atoms, res.fatm[0] + i, FA->bloops, &nbonded, bondlist.data(), neighbours.data());
                update_bonded(&res, na, nbonded, bondlist.data(), neighbours.data());
            }
            FA->flex_res[r].inum = kres;
            FA->flex_res[r].num = res.number;
            FA->flex_res[r].chn = res.chn;
            FA->flex_res[r].prob = 1.0f;
            FA->flex_res[r].cflag = 1;
            strcpy(FA->flex_res[r].name, res.name);
            for (int k = 0; k < na; ++k)
                if (!in->flex_isbb[isbb_off[r] + k]) h.sc_slot.push_back(in->flex_first[r] + k);
        }
        FA->num_optres = 1 + in->n_flexres;
        FA->nflxsc = in->n_flexres;
        FA->nflxsc_real = in->n_flexres;
    }

    // cleft grid: entry 0 is the initial ligand anchor (LIB/generate_grid.cpp:26-30)
    h.cleftgrid = (gridpoint*)calloc(in->n_grid + 1, sizeof(gridpoint));
    gridpoint* cg = h.cleftgrid;
    const int g0 = lr.gpa[0];
    for (int j = 0; j < 3; ++j) cg[0].coor[j] = atoms[g0].coor[j];
    cg[0].dis = atoms[g0].dis;
    cg[0].ang = atoms[g0].ang;
    cg[0].dih = atoms[g0].dih;
    for (int i = 0; i < in->n_grid; ++i) {
        cg[i + 1].number = i + 1;
        for (int j = 0; j < 3; ++j) cg[i + 1].coor[j] = in->grid_xyz[i * 3 + j];
    }
    FA->num_grd = in->n_grid + 1;
    calc_cleftic(FA, cg);
    ic_bounds(FA, FA->rngopt);

    // genes: translation, rotation, flexible bonds (LIB/top.cpp:968-985)
    int opt[2];
    opt[0] = lr.number;
    opt[1] = -1;
    add2_optimiz_vec(FA, atoms, residue, opt, ' ', "");
    opt[1] = 0;
    add2_optimiz_vec(FA, atoms, residue, opt, ' ', "");
    for (int j = 1; j <= lr.fdih; ++j) {
        opt[1] = j;
        add2_optimiz_vec(FA, atoms, residue, opt, ' ', "");
    }
    if (in->n_flexres > 0) add2_optimiz_vec(FA, atoms, residue, opt, ' ', "SC");
    update_optres(atoms, residue, FA->atm_cnt, FA->optres, FA->num_optres);

    // energy matrix (LIB/read_emat.cpp:56-126 layout)
    const int T = in->ntypes;
    FA->ntypes = T;
    FA->energy_matrix = (struct energy_matrix*)calloc((size_t)T * T, sizeof(struct energy_matrix));
    for (int i = 0; i < T; ++i)
        for (int j = 0; j < T; ++j) {
            struct energy_matrix& em = FA->energy_matrix[i * T + j];
            em.type1 = i + 1;
            em.type2 = j + 1;
            const int idx = i * T + j;
            em.weight = in->emat_weight[idx];
            struct energy_values* prev = nullptr;
            for (int p = in->emat_off[idx]; p < in->emat_off[idx + 1]; ++p) {
                auto* v = (struct energy_values*)malloc(sizeof(struct energy_values));
                v->x = in->emat_x[p];
                v->y = in->emat_y[p];
                v->next_value = nullptr;
                if (prev) prev->next_value = v; else em.energy_values = v;
                prev = v;
            }
        }
    FA->contributions = (float*)calloc((size_t)T * T, sizeof(float));

    // Vcontacts allocations (LIB/top.cpp:1011-1043)
    VC->planedef = FA->vcontacts_planedef;
    VC->Calc = (atomsas*)calloc(FA->atm_cnt_real, sizeof(atomsas));
    VC->Calclist = (int*)malloc(FA->atm_cnt_real * sizeof(int));
    VC->ca_index = (int*)malloc(FA->atm_cnt_real * sizeof(int));
    VC->seed = (int*)malloc(3 * FA->atm_cnt_real * sizeof(int));
    VC->contlist = (contactlist*)malloc(10000 * sizeof(contactlist));
    VC->ca_recsize = 5 * FA->atm_cnt_real;
    VC->ca_rec = (ca_struct*)malloc(VC->ca_recsize * sizeof(ca_struct));
    for (int i = 0; i < FA->atm_cnt_real; ++i) {
        VC->Calc[i].atom = nullptr;
        VC->Calc[i].residue = nullptr;
        VC->Calc[i].exposed = true;
    }
    FA->deelig_root_node = new struct deelig_node_struct;
    FA->deelig_root_node->parent = nullptr;

    create_rebuild_list(FA, atoms, residue);
    // first evaluation at the initial conformation, then no hull recalculation
    ic2cf(FA, VC, atoms, residue, cg, FA->npar, FA->opt_par);
    VC->recalc = 0;
    return 0;
}

int ref_sizes(ref_export_sizes* s) {
    if (!H) return -1;
    s->n_atoms = H->FA->atm_cnt_real;
    s->n_lig = H->n_lig;
    s->n_genes = H->FA->npar;
    s->n_grid = H->FA->num_grd;
    s->n_mov = H->FA->nmov[0];
    return 0;
}

// Exports the set-up state the evaluation reads, in ligand-local numbering.
int ref_export(float* ori, float* gmin, float* gmax, float* maxwidth,
               float* grid_ic,             // n_grid * 3
               float* lig_ic,              // n_lig * 3 (dis, ang, dih)
               float* lig_shift,           // n_lig
               int32_t* lig_rec,           // n_lig * 4, -1 = reference frame / no cycle
               int32_t* mov,               // n_mov
               int8_t* bonded,             // n_lig * n_lig
               int32_t* gene_typ, int32_t* gene_atm,
               double* gene_min, double* gene_max, double* gene_del, int32_t* gene_map,
               double* opt_par) {
    if (!H) return -1;
    Harness& h = *H;
    FA_Global* FA = h.FA;
    for (int j = 0; j < 3; ++j) {
        ori[j] = FA->ori[j];
        gmin[j] = FA->globalmin[j];
        gmax[j] = FA->globalmax[j];
    }
    *maxwidth = FA->maxwidth;
    for (int i = 0; i < FA->num_grd; ++i) {
        grid_ic[i * 3 + 0] = h.cleftgrid[i].dis;
        grid_ic[i * 3 + 1] = h.cleftgrid[i].ang;
        grid_ic[i * 3 + 2] = h.cleftgrid[i].dih;
    }
    const int N = h.n_rec, n = h.n_lig;
    for (int i = 0; i < n; ++i) {
        const atom& a = h.atoms[N + 1 + i];
        lig_ic[i * 3 + 0] = a.dis;
        lig_ic[i * 3 + 1] = a.ang;
        lig_ic[i * 3 + 2] = a.dih;
        lig_shift[i] = a.shift;
        for (int j = 0; j < 4; ++j) lig_rec[i * 4 + j] = to_local(h, a.rec[j]);
    }
    for (int i = 0; i < FA->nmov[0]; ++i) mov[i] = to_local(h, FA->mov[0][i]);
    resid& lr = h.residue[h.lig_res];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) bonded[i * n + j] = (int8_t)lr.bonded[i][j];
    for (int g = 0; g < FA->npar; ++g) {
        gene_typ[g] = FA->map_par[g].typ;
        gene_atm[g] = to_local(h, FA->map_par[g].atm);
        if (FA->map_par[g].typ == 4)   // the flexible side chain, by its place in FA->flex_res
            for (int r = 0; r < FA->nflxsc; ++r)
                if (h.residue[FA->flex_res[r].inum].fatm[0] == FA->map_par[g].atm) gene_atm[g] = r;
        gene_min[g] = FA->min_opt_par[g];
        gene_max[g] = FA->max_opt_par[g];
        gene_del[g] = FA->del_opt_par[g];
        gene_map[g] = FA->map_opt_par[g];
        opt_par[g] = FA->opt_par[g];
    }
    return 0;
}

// The bonded matrices of the flexible side chains (natm * natm each, concatenated in order).
int ref_export_flex_bonded(int8_t* out) {
    if (!H) return -1;
    Harness& h = *H;
    size_t o = 0;
    for (int r = 0; r < h.FA->nflxsc; ++r) {
        const resid& res = h.residue[h.FA->flex_res[r].inum];
        const int na = res.latm[0] - res.fatm[0] + 1;
        for (int i = 0; i < na; ++i)
            for (int j = 0; j < na; ++j) out[o++] = (int8_t)res.bonded[i][j];
    }
    return (int)o;
}

// Evaluates n chromosomes given as decoded ICs (n * n_genes doubles). cf_out holds, per pose,
// com, con, wal, sas, elec, gist, hbond, gist_desolv, metal_coord, evalue, rclash.
// status_out: 0 scored, 1 polyhedron failure, 2 clash pre-filter rejection.
int ref_eval(int32_t n, const double* ic, double* cf_out, int32_t* status_out,
             float* lig_xyz_out /* n * n_lig * 3, or NULL */) {
    if (!H) return -1;
    Harness& h = *H;
    FA_Global* FA = h.FA;
    const int ng = FA->npar;
    std::vector<double> icv(ng > 0 ? ng : 1);
    for (int p = 0; p < n; ++p) {
        for (int g = 0; g < ng; ++g) {
            double v = ic[(size_t)p * ng + g];
            if (v > FA->max_opt_par[g]) v = FA->max_opt_par[g];
            else if (v < FA->min_opt_par[g]) v = FA->min_opt_par[g];
            icv[g] = v;
        }
        const int sk = FA->skipped, cl = FA->clashed;
        // order_faces (LIB/Vcontacts.cpp:800-812) can read ptorder[X].pt[numpts], a slot no
        // code path writes before reading when a face has no vertex on its second plane; the
        // caller-owned workspace is zeroed before every pose so that such reads are defined.
        memset(h.VC->ptorder, 0, MAX_PT * sizeof(ptindex));
        // voronoi_poly2 answers a hull walk of 200 edges by moving the atom by a random
        // +-0.005 A and, on this path (VC->recalc = 0), does not move it back
        // (LIB/Vcontacts.cpp:378-405, 480-487). Ligand atoms are rebuilt every pose; rotamer
        // atoms are not, so the displacement would stay with every later pose. The rotamer
        // coordinates are put back before each pose so that poses do not depend on the ones
        // evaluated before them.
        for (const auto& ra : h.rotamer_atoms)
            for (int c = 0; c < 3; ++c) h.atoms[ra.first].coor[c] = ra.second[c];
        cfstr cf = ic2cf(FA, h.VC, h.atoms, h.residue, h.cleftgrid, ng, icv.data());
        double* o = cf_out + (size_t)p * 11;
        o[0] = cf.com; o[1] = cf.con; o[2] = cf.wal; o[3] = cf.sas; o[4] = cf.elec;
        o[5] = 0.0;  // cf.gist is left unset by ic2cf on the success path
        o[6] = cf.hbond; o[7] = cf.gist_desolv; o[8] = cf.metal_coord;
        o[9] = get_cf_evalue(&cf);
        o[10] = cf.rclash;
        status_out[p] = FA->skipped != sk ? 1 : (FA->clashed != cl ? 2 : 0);
        if (lig_xyz_out)
            for (int i = 0; i < h.n_lig; ++i)
                for (int j = 0; j < 3; ++j)
                    lig_xyz_out[((size_t)p * h.n_lig + i) * 3 + j] = h.atoms[h.n_rec + 1 + i].coor[j];
        // contact records of the scored atoms: side-chain atoms, then the ligand (whose Calc
        // indices follow the receptor's)
        const int nsc = (int)h.sc_slot.size(), ns = nsc + h.n_lig;
        h.last_contacts.assign(ns, {});
        h.last_areas.assign(ns, {});
        h.last_dists.assign(ns, {});
        if (status_out[p] == 0) {
            for (int i = 0; i < ns; ++i) {
                int ci = h.VC->ca_index[i < nsc ? h.sc_slot[i] : h.n_rec + (i - nsc)];
                while (ci != -1) {
                    h.last_contacts[i].push_back(h.VC->ca_rec[ci].atom);
                    h.last_areas[i].push_back(h.VC->ca_rec[ci].area);
                    h.last_dists[i].push_back(h.VC->ca_rec[ci].dist);
                    ci = h.VC->ca_rec[ci].prev;
                }
            }
        }
    }
    return 0;
}

// Contact records of the last evaluated pose for scored atom i (side-chain atoms first, then the
// ligand), in record-walk order.
int ref_last_contacts(int32_t i, int32_t cap, int32_t* partner, double* area, double* dist) {
    if (!H || i < 0 || i >= (int)H->last_contacts.size()) return -1;
    const auto& c = H->last_contacts[i];
    const int m = (int)c.size();
    for (int k = 0; k < m && k < cap; ++k) {
        partner[k] = c[k];
        area[k] = H->last_areas[i][k];
        dist[k] = H->last_dists[i][k];
    }
    return m;
}

// Runs the reference's CF-based clustering (cluster, LIB/cluster.cpp:9-182) over n chromosomes
// given as ICs (n * n_genes, within their gene limits) and their app_evalue, with
// FA->temperature, FA->beta (1 / temperature, as read_input sets it), FA->cluster_rmsd and
// FA->max_results as given. The reference writes <prefix>.cad (cluster table and the RMSD between
// cluster heads) and <prefix>_<k>.pdb per result, which the tests read.
int ref_cluster(int32_t n, const double* ic, const double* app_evalue, int32_t temperature, float rmsd,
                int32_t max_results, const char* prefix) {
    if (!H || n < 1 || !prefix || strlen(prefix) + 16 >= MAX_PATH__) return -1;
    Harness& h = *H;
    FA_Global* FA = h.FA;
    const int ng = FA->npar;
    GB_Global GB{};
    GB.num_genes = ng;
    std::vector<chromosome> chrom(n);
    std::vector<gene> genes((size_t)n * ng);
    for (int p = 0; p < n; ++p) {
        chrom[p] = chromosome{};
        chrom[p].genes = &genes[(size_t)p * ng];
        for (int g = 0; g < ng; ++g) genes[(size_t)p * ng + g].to_ic = ic[(size_t)p * ng + g];
        chrom[p].evalue = chrom[p].app_evalue = app_evalue[p];
    }
    std::vector<genlim> lim(ng > 0 ? ng : 1);
    for (int g = 0; g < ng; ++g) {
        lim[g].min = FA->min_opt_par[g];
        lim[g].max = FA->max_opt_par[g];
        lim[g].del = FA->del_opt_par[g];
        lim[g].map = FA->map_opt_par[g];
    }
    FA->temperature = (uint)temperature;
    FA->beta = temperature > 0 ? (double)(1.0 / FA->temperature) : 0.0;
    FA->cluster_rmsd = rmsd;
    FA->max_results = max_results;
    FA->htpmode = false;
    FA->refstructure = 0;
    FA->het_res[1] = h.lig_res;   // the ligand residue (write_pdb's CONECT records)
    char end_strfile[MAX_PATH__], tmp_end_strfile[MAX_PATH__], dockinp[] = "dock.inp", gainp[] = "ga.inp";
    snprintf(end_strfile, sizeof(end_strfile), "%s", prefix);
    for (const auto& ra : h.rotamer_atoms)
        for (int c = 0; c < 3; ++c) h.atoms[ra.first].coor[c] = ra.second[c];
    cluster(FA, &GB, h.VC, chrom.data(), lim.data(), h.atoms, h.residue, h.cleftgrid, n, end_strfile,
            tmp_end_strfile, dockinp, gainp);
    FA->htpmode = true;
    FA->temperature = 0;
    FA->beta = 0.0;
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// The C++ adapter's packing (flexaidds_gb300/adapter/fxe_flexaid_pack.cpp) of this harness's
// state, for the check that it packs what the reference's set-up produced.
// ---------------------------------------------------------------------------------------------
#include "fxe_flexaid.h"

namespace {
FxeFlexaidPacked g_packed;
}

extern "C" {

// Packs the harness state; sizes[0..6] = receptor atoms, grid entries, ligand atoms, genes,
// rebuild-list length, energy-matrix points, flexible side chains. Returns 0, or -1 with the
// adapter's message in msg (cap bytes).
int ref_adapter_pack(int32_t* sizes, char* msg, int32_t cap) {
    if (!H) return -1;
    std::string err;
    if (!fxe_flexaid_pack(H->FA, H->atoms, H->residue, H->cleftgrid, &g_packed, &err)) {
        if (msg && cap > 0) snprintf(msg, (size_t)cap, "%s", err.c_str());
        return -1;
    }
    const FxeFlexaidPacked& P = g_packed;
    sizes[0] = P.receptor.n_atoms;
    sizes[1] = P.receptor.n_grid;
    sizes[2] = P.ligand.n_atoms;
    sizes[3] = P.ligand.n_genes;
    sizes[4] = P.ligand.n_build;
    sizes[5] = (int32_t)P.em_x.size();
    sizes[6] = P.receptor.n_flex;
    return 0;
}

// Copies one packed array by name into dst (sized by the caller from ref_adapter_pack's sizes).
// Scalars: "frame" = ori, globalmin, globalmax, maxwidth (10 floats); "params" = permeability,
// dee_clash, intramolecular, solventterm (4 floats). Flexible side chain r: "flex_info" (4 ints per
// chain: first, atoms, rotamers, 0), "flex_backbone", "flex_xyz", "flex_bonded" concatenated.
int ref_adapter_get(const char* name, void* dst) {
    const FxeFlexaidPacked& P = g_packed;
    const std::string k(name);
    auto put = [&](const auto& v) {
        memcpy(dst, v.data(), v.size() * sizeof(v[0]));
        return (int)v.size();
    };
    if (k == "rec_xyz") return put(P.rec_xyz);
    if (k == "rec_radius") return put(P.rec_radius);
    if (k == "rec_type") return put(P.rec_type);
    if (k == "grid_ic") return put(P.grid_ic);
    if (k == "lig_radius") return put(P.lig_radius);
    if (k == "lig_type") return put(P.lig_type);
    if (k == "lig_rec") return put(P.lig_rec);
    if (k == "lig_shift") return put(P.lig_shift);
    if (k == "lig_ic") return put(P.lig_ic);
    if (k == "build_order") return put(P.build_order);
    if (k == "bonded") return put(P.bonded);
    if (k == "gene_typ") return put(P.gene_type);
    if (k == "gene_atm") return put(P.gene_atom);
    if (k == "gene_min") return put(P.gene_min);
    if (k == "gene_max") return put(P.gene_max);
    if (k == "gene_del") return put(P.gene_del);
    if (k == "gene_map") return put(P.gene_map);
    if (k == "emat_weight") return put(P.em_weight);
    if (k == "emat_off") return put(P.em_offset);
    if (k == "emat_x") return put(P.em_x);
    if (k == "emat_y") return put(P.em_y);
    if (k == "frame") {
        float* f = static_cast<float*>(dst);
        for (int c = 0; c < 3; ++c) {
            f[c] = P.receptor.ori[c];
            f[3 + c] = P.receptor.globalmin[c];
            f[6 + c] = P.receptor.globalmax[c];
        }
        f[9] = P.receptor.maxwidth;
        return 10;
    }
    if (k == "params") {
        float* f = static_cast<float*>(dst);
        f[0] = P.params.permeability;
        f[1] = P.params.dee_clash;
        f[2] = (float)P.params.intramolecular;
        f[3] = P.params.solventterm;
        return 4;
    }
    if (k == "flex_info") {
        int32_t* o = static_cast<int32_t*>(dst);
        for (size_t r = 0; r < P.flex.size(); ++r) {
            o[4 * r] = P.flex[r].first;
            o[4 * r + 1] = P.flex[r].n_atoms;
            o[4 * r + 2] = P.flex[r].n_rot;
            o[4 * r + 3] = 0;
        }
        return (int)(4 * P.flex.size());
    }
    auto cat = [&](const auto& vv) {
        size_t o = 0;
        for (const auto& v : vv) {
            memcpy(static_cast<char*>(dst) + o * sizeof(v[0]), v.data(), v.size() * sizeof(v[0]));
            o += v.size();
        }
        return (int)o;
    };
    if (k == "flex_backbone") return cat(P.flex_backbone);
    if (k == "flex_xyz") return cat(P.flex_xyz);
    if (k == "flex_bonded") return cat(P.flex_bonded);
    return -1;
}

}  // extern "C"
