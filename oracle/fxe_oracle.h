/* fxe_oracle.h — CPU restatement of the FlexAID∆S fitness-evaluation path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker the GPU path is compared against (tests/,
 * the smoke check, and the bench's CPU-baseline leg). The product never links or calls it.
 *
 * Parity is pinned: tests compare this restatement with the reference's own code compiled
 * from its sources (oracle/_ref) on seeded systems, pose for pose, and with the golden
 * fixtures generated from that reference (tests/golden/).
 */
#ifndef FXE_ORACLE_H
#define FXE_ORACLE_H

#include "../include/fxe.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One recorded contact of a scored pose (a ca_rec entry walked by vcfunction). */
typedef struct fxo_contact {
    int32_t pose;
    int32_t atom;      /* ligand-local index of the scorable atom */
    int32_t partner;   /* Calc index of the contact partner */
    float area;
    float dist;
} fxo_contact;

/* Work counters per scorable atom, summed over the poses of one call (the algorithmic
 * counts behind the FLOP model): candidates scanned, contacts, polyhedron edges walked,
 * edges tested for arc points, spherical triangles + arc segments, polyhedron vertices. */
typedef struct fxo_counts {
    int64_t atoms, candidates, contacts, edges, arc_edges, triangles, vertices, built_atoms;
    int64_t no_partner;  /* faces whose first vertex has no neighbour on its second plane */
    int64_t plane_tests; /* sum over atoms of contacts x hull edges walked */
} fxo_counts;

/* Reference-compat mode: reproduce the reference's read of the slot past a face's vertex list
 * in order_faces (see fxe_oracle.c), on a workspace zeroed at the start of every pose. Used
 * only to pin this restatement against the compiled reference; off by default. */
void fxo_set_reference_compat(int on);

/* 0 (default): cosf/sinf of the C library in the pose build, as the reference;
   1: correctly rounded single-precision cos/sin. */
void fxo_set_trig_rounding(int correctly_rounded);

/* Scores n poses given as decoded ICs (n * n_genes). xyz_out (n * n_lig * 3) receives the
 * built ligand coordinates when non-NULL; contacts_out (capacity cap) the recorded contacts,
 * their number through *n_contacts; counts accumulates the work counters when non-NULL.
 * Returns 0, or -1 on invalid input. */
int fxo_eval_ic(const fxe_receptor_desc* rec, const fxe_ligand_desc* lig,
                const fxe_emat_desc* emat, const fxe_params* prm, int32_t n, const double* ic,
                fxe_cf* out, float* xyz_out, fxo_contact* contacts_out, int64_t cap,
                int64_t* n_contacts, fxo_counts* counts);

/* Decodes n chromosomes of int32 genes to ICs as genetoic does. */
int fxo_genes_to_ic(const fxe_ligand_desc* lig, int32_t n, const int32_t* genes, double* ic);

/* FP64 canonical-ensemble thermodynamics (StatMechEngine::compute). */
int fxo_thermo(const double* e, const int32_t* mult, int64_t n, double temperature,
               fxe_thermo* out);
int fxo_thermo_weights(const double* e, const int32_t* mult, int64_t n, double temperature,
                       double* w);

/* Ligand coordinates of n chromosomes given as ICs, as calc_rmsd_chrom builds them (no clamp);
 * xyz_out n * n_lig * 3. */
int fxo_build_ic(const fxe_receptor_desc* rec, const fxe_ligand_desc* lig, int32_t n, const double* ic,
                 float* xyz_out);

/* CF-based clustering (cluster, LIB/cluster.cpp:9-218), serial, with the reference's order of
 * sums; arguments and outputs as fxe_cluster. Returns 0, -1 (invalid input) or -2 (zero
 * partition function). */
int fxo_cluster(const fxe_receptor_desc* rec, const fxe_ligand_desc* lig, int32_t n, const double* ic,
                const double* app_evalue, int32_t temperature, float rmsd_threshold, int32_t max_results,
                int32_t* top, int32_t* freq, double* tcf, double* acf, int32_t* member_of, float* rmsd,
                float* top_rmsd, int32_t* n_clusters);

/* Geometry helpers restated from LIB/Vcontacts.cpp, exported for known-answer tests. */
int fxo_solve_3x3(const double* eq0, const double* eq1, const double* eq2, double* pt);
int fxo_solve_2xS(const double* p0, const double* p1, float rado, double* pt0, double* pt1);
double fxo_cosPQR(const double* p, const double* q, const double* r);
double fxo_spherical_arc(const double* ao, double ao_dist, const double* b, double b_dist,
                         const double* c, double c_dist, float rado);

#ifdef __cplusplus
}
#endif

#endif
