/* fxe.h — C ABI of the GB300 fitness-evaluation backend for FlexAID∆S-style docking.
 *
 * One call scores a batch of chromosomes: gene decode -> pose build -> receptor cell list ->
 * Voronoi contact surfaces -> energy-matrix complementarity with wall/clash terms, returning
 * the reference's complementarity-function record (cfstr) per pose; a second entry point
 * reduces an ensemble of pose energies to its canonical-ensemble thermodynamics in FP64.
 *
 * Plain C: plain pointers and sizes, status codes, no exceptions cross this boundary.
 * All entry points are thread-safe except that one fxe_context must not be used by two
 * threads at once (it owns one CUDA stream).
 */
#ifndef FXE_H
#define FXE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes; mirror hw::DispatchError (LIB/UnifiedHardwareDispatch.h:63-72) in place of
 * the exceptions the reference's CUDA backend throws from CUDA_CHECK
 * (LIB/cuda_eval.cu:38-45, 318-326). */
typedef enum fxe_status {
    FXE_OK = 0,
    FXE_ERR_INVALID_ARGS = 1,
    FXE_ERR_ALLOC = 2,
    FXE_ERR_LAUNCH = 3,
    FXE_ERR_TIMEOUT = 4,
    FXE_ERR_OVER_BUDGET = 5,
    FXE_ERR_CAPACITY = 6,   /* a pose exceeded a fixed per-atom capacity; see fxe_cf.status */
    FXE_ERR_NO_DEVICE = 7,
    FXE_ERR_INTERNAL = 8
} fxe_status;

/* A flexible side chain: a receptor residue with rotamers (LIB/build_rotamers.cpp). Its atoms
 * are receptor atoms first .. first + n_atoms - 1 (Calc order). The residue's rotamer gene
 * (gene type 4, gene_atom = the residue's index in fxe_receptor_desc.flex) selects rotamer
 * r = (unsigned)(ic + 0.5) (LIB/ic2cf.cpp:90-94), whose coordinates the residue's atoms then
 * take; rotamer 0 is the receptor's own conformation. Its non-backbone atoms are scored like
 * ligand atoms (update_optres, LIB/update_optres.cpp:17-28), each residue with its own
 * complementarity record summed after the ligand's (LIB/ic2cf.cpp:133-245). */
typedef struct fxe_flex_residue {
    int32_t first;
    int32_t n_atoms;
    int32_t n_rot;             /* rotamers, including rotamer 0 */
    const int8_t* backbone;    /* n_atoms: 1 = backbone atom (keeps its place, not scored) */
    const float* rot_xyz;      /* n_rot * n_atoms * 3 */
    const int8_t* bonded;      /* n_atoms * n_atoms: residue.bonded (-1: not within bloops) */
    float prob;                /* flxsc.prob, for the GA engine: the chance that a child's rotamer
                                  gene mutates and that an initial chromosome draws one (else
                                  rotamer 0) (LIB/gaboom.cpp:944-966, 1875-1895; the reference's
                                  per-residue defaults are set_intprob's, LIB/set_intprob.cpp) */
} fxe_flex_residue;

/* Receptor, in the reference's Calc order (residue order, LIB/Vcontacts.cpp:1600-1630),
 * plus the state LIB/calc_center.cpp:8-61 leaves in FA and the cleft grid of
 * LIB/generate_grid.cpp / LIB/calc_cleftic.cpp. */
typedef struct fxe_receptor_desc {
    int32_t n_atoms;
    const float* xyz;          /* n_atoms * 3 */
    const float* radius;       /* n_atoms */
    const int32_t* type;       /* n_atoms, 1..ntypes */
    float ori[3];              /* FA->ori: frame origin for unreferenced build atoms */
    float globalmin[3];        /* FA->globalmin */
    float globalmax[3];        /* FA->globalmax */
    float maxwidth;            /* FA->maxwidth */
    int32_t n_grid;            /* cleft grid entries including entry 0 (initial anchor) */
    const float* grid_ic;      /* n_grid * 3: dis, ang, dih of each grid point */
    int32_t n_flex;            /* flexible side chains (0..8; at most 32 scored atoms in all) */
    const fxe_flex_residue* flex;
} fxe_receptor_desc;

/* Ligand build tree and genes (atoms/residue/FA->map_par after the reference set-up:
 * LIB/read_lig.cpp, LIB/assign_shift.cpp, LIB/add2_optimiz_vec.cpp, LIB/create_rebuild_list.cpp).
 * Atom indices are ligand-local (0..n_atoms-1); -1 stands for the reference frame
 * (rec == 0 in the reference) or, in rec[3], for "no dihedral cascade". */
typedef struct fxe_ligand_desc {
    int32_t n_atoms;
    const float* radius;       /* n_atoms */
    const int32_t* type;       /* n_atoms */
    const int32_t* rec;        /* n_atoms * 4: rec[0..2] build references, rec[3] cascade */
    const float* shift;        /* n_atoms: dihedral shift along the rec[3] cycle */
    const float* ic;           /* n_atoms * 3: base dis, ang, dih */
    int32_t n_build;
    const int32_t* build_order;/* n_build: FA->mov[0] */
    const int8_t* bonded;      /* n_atoms * n_atoms: residue.bonded (-1: not within bloops) */
    int32_t n_genes;
    const int32_t* gene_type;  /* optmap.typ: -1 grid index, 0 dis, 1 ang, 2 dih, 4 rotamer */
    const int32_t* gene_atom;  /* optmap.atm, ligand-local; for a rotamer gene the residue */
    const double* gene_min;    /* genlim.min / max / del / map (LIB/gaboom.cpp:2491-2507) */
    const double* gene_max;
    const double* gene_del;
    const int32_t* gene_map;
} fxe_ligand_desc;

/* Energy matrix (LIB/flexaid.h:155-166, read by LIB/read_emat.cpp): per ordered type pair a
 * weight flag and a piecewise-linear curve; single-valued (weight = 1) entries use curve_y of
 * their one point. */
typedef struct fxe_emat_desc {
    int32_t ntypes;
    const int32_t* weight;     /* ntypes * ntypes */
    const int32_t* offset;     /* ntypes * ntypes + 1 */
    const float* x;
    const float* y;
} fxe_emat_desc;

/* Scoring switches read by LIB/vcfunction.cpp (FA->permeability, dee_clash, intramolecular,
 * solventterm). The optional terms (useacs, normalize_area, electrostatics, H-bonds, GIST,
 * metal coordination, constraints) are off, as in the reference defaults (LIB/top.cpp:233-330). */
typedef struct fxe_params {
    float permeability;
    float dee_clash;
    int32_t intramolecular;
    float solventterm;
} fxe_params;

/* Per-pose outcome: the reference's cfstr (LIB/flexaid.h:122-135) plus the evalue of
 * get_cf_evalue (LIB/ic2cf.cpp:396-401) and how the pose ended. */
typedef struct fxe_cf {
    double com, con, wal, sas, elec, gist, hbond, gist_desolv, metal_coord, totsas;
    double evalue;
    int32_t rclash;
    int32_t status;            /* FXE_POSE_* */
} fxe_cf;

enum {
    FXE_POSE_SCORED = 0,
    FXE_POSE_POLYHEDRON_FAILED = 1, /* LIB/vcfunction.cpp:68-71: wal = 1e6 */
    FXE_POSE_CLASHED = 2,           /* LIB/vcfunction.cpp:72-74: wal = clash sum >= 1e4 */
    FXE_POSE_CAPACITY = 3           /* exceeded a fixed per-atom workspace; not scored */
};

/* Canonical-ensemble thermodynamics (LIB/statmech.h:36-48, LIB/statmech.cpp:73-174). */
typedef struct fxe_thermo {
    double temperature, log_Z, free_energy, mean_energy, mean_energy_sq, heat_capacity,
           entropy, std_energy;
} fxe_thermo;

/* Receptor preparation on the device: the cleft grid of generate_grid
 * (LIB/generate_grid.cpp:18-107) and its internal coordinates (calc_cleftic,
 * LIB/calc_cleftic.cpp:5-33), the fxe_receptor_desc grid entries 1.. (entry 0, the ligand's
 * initial anchor, is the caller's). Spheres (centres n_spheres * 3, radii) are walked in the
 * order given, as generate_grid walks its sphere list: the lattice of each (steps of `spacing`
 * from the reference's rounded lower bound, x fastest) keeps the points strictly inside the
 * sphere, and a point whose coordinates, snapped to 0.001 A (GridKey, LIB/maps.hpp:21-49),
 * match a point of an earlier sphere is dropped. ICs against the frame ori + (1,0,0), ori,
 * ori + (0,1,0) in single precision; the bond angle and dihedral round the double-precision
 * acos and atan2, where the reference calls the C library's acosf and atan2f, so about one
 * value in five can differ from the reference's in the last bit. xyz and ic: cap * 3 floats
 * (host; ic may be NULL); *n_points the count (FXE_ERR_CAPACITY when it exceeds cap: call with
 * cap 0 to size). Centres within +-1000 A, radii in (0, 1000]. */
fxe_status fxe_cleft_grid(int32_t n_spheres, const float* centers, const float* radii, float spacing,
                          const float* ori, int64_t cap, float* xyz, float* ic, int64_t* n_points);

typedef struct fxe_context fxe_context;

/* Creates an evaluation context on the current CUDA device: copies the descriptors into
 * device memory, builds the receptor cell list (on the device) and the gene decode tables, and reserves
 * workspace for up to max_poses poses per call. Replaces cuda_eval_init
 * (LIB/cuda_eval.cuh:46-58) and GPUContextPool::acquire_cuda (LIB/GPUContextPool.h:56-100). */
fxe_status fxe_context_create(const fxe_receptor_desc* receptor, const fxe_ligand_desc* ligand,
                              const fxe_emat_desc* emat, const fxe_params* params,
                              int32_t max_poses, fxe_context** out);

/* A context for another ligand (or energy matrix, or scoring switches) on the receptor of
 * `receptor_of`: the receptor atoms, cell list and cleft grid stay where `receptor_of` put them
 * and are shared, not copied (the receptor cache); they live until the last context using them
 * is destroyed. No reference counterpart: the reference keeps one receptor per process. */
fxe_status fxe_context_create_shared(const fxe_context* receptor_of, const fxe_ligand_desc* ligand,
                                     const fxe_emat_desc* emat, const fxe_params* params,
                                     int32_t max_poses, fxe_context** out);

/* Arithmetic of the Voronoi polyhedra and contact areas.
 * FXE_PRECISION_REFERENCE (default): double precision with the reference's own expressions and
 *   no fused multiply-adds, so that every operation rounds as in the reference's double
 *   arithmetic; the reference's areas are sensitive to last-bit rounding on degenerate faces
 *   (coincident projected vertices, antipodal arc points), and this mode reproduces them.
 * FXE_PRECISION_FAST: single precision with well-conditioned equivalents of the area
 *   expressions; agrees with the reference to about 1e-6 on typical poses and differs where the
 *   reference's result is decided by rounding. */
enum { FXE_PRECISION_REFERENCE = 0, FXE_PRECISION_FAST = 1 };
fxe_status fxe_context_set_precision(fxe_context* ctx, int32_t precision);

/* How a face whose first point has no other point on its second plane is ordered. order_faces
 * (LIB/Vcontacts.cpp:800-812) then swaps point 1 with ptorder[X].pt[numpts], a slot past the
 * face's own list that holds what an earlier atom of the pose left there.
 * FXE_FACE_ORDER_REFERENCE (default): that read is replayed as the reference makes it on a
 *   ptorder workspace cleared at the start of each pose: the device keeps each contact's last
 *   point list for the pose (faces of at most 63 points; a longer one is counted in
 *   fxe_last_stats out4[0] and ordered as below).
 * FXE_FACE_ORDER_GEOMETRIC: point 1 is the first point sharing the first point's other plane, a
 *   neighbour on the face, so the face's points are ordered by angle as the reference intends.
 * Batched launches and the GA engine use the reference order unless every context of the launch
 * asks for the geometric one; the GA engine reads the setting when its set of running jobs
 * changes. No reference counterpart (the reference has no switch). */
enum { FXE_FACE_ORDER_REFERENCE = 0, FXE_FACE_ORDER_GEOMETRIC = 1 };
fxe_status fxe_context_set_face_order(fxe_context* ctx, int32_t mode);

/* How the contact-candidate scan reads the receptor's cell list. The scan of an atom's 27
 * neighbouring cells (get_contlist4, LIB/Vcontacts.cpp:1725-1839) takes their rigid entries
 * FXE_CELLS_IN_PLACE: from global memory where they lie (through L1 and L2);
 * FXE_CELLS_STAGED: from shared memory, staged first by bulk copies (one cp.async.bulk per row of
 *   three neighbouring cells, which lie together in the cell list) when the 27 cells hold at most
 *   256 entries, in place otherwise;
 * FXE_CELLS_AUTO (default): the form fxe_context_autotune measured faster for the launch's size
 *   class, in place when the class is not tuned.
 * Results are the same in every form. Batched launches and the GA engine use the contexts' common
 * setting, else AUTO. No reference counterpart. */
enum { FXE_CELLS_AUTO = 0, FXE_CELLS_IN_PLACE = 1, FXE_CELLS_STAGED = 2 };
fxe_status fxe_context_set_cell_staging(fxe_context* ctx, int32_t mode);

/* Scores n chromosomes given as int32 genes (n * n_genes, host memory), writing n records to
 * host memory. Synchronous, like cuda_eval_batch (LIB/cuda_eval.cuh:60-70). */
fxe_status fxe_eval_genes(fxe_context* ctx, int32_t n, const int32_t* genes, fxe_cf* out);

/* Same, for chromosomes given as decoded internal coordinates (n * n_genes doubles), the
 * icv vector that eval_chromosome hands to ic2cf (LIB/gaboom.cpp:1845-1866). */
fxe_status fxe_eval_ic(fxe_context* ctx, int32_t n, const double* ic, fxe_cf* out);

/* Device-resident form: genes and out are device pointers; work is queued on `stream`
 * (a cudaStream_t, or NULL for the context's own stream) and not waited for. */
fxe_status fxe_eval_genes_device(fxe_context* ctx, int32_t n, const int32_t* d_genes,
                                 fxe_cf* d_out, void* stream);

/* Contacts recorded for the last evaluated batch (the ca_rec lists vcfunction walks), for
 * inspection and parity checks: for pose p and scored atom a, up to cap entries of
 * (partner Calc index, area). Scored atoms are the flexible side chains' non-backbone atoms in
 * Calc order, then the ligand atoms (without side chains: a is the ligand atom). Returns the
 * count through *n_out. */
fxe_status fxe_last_contacts(fxe_context* ctx, int32_t pose, int32_t atom, int32_t cap,
                             int32_t* partner, float* area, int32_t* n_out);

/* Built ligand coordinates of pose `pose` of the last evaluated batch (n_atoms * 3). */
fxe_status fxe_last_ligand_xyz(fxe_context* ctx, int32_t pose, float* xyz);

/* Work counters of the last evaluation call: out4[0] faces whose read past the end of their
 * point list could not be replayed (FXE_FACE_ORDER_REFERENCE; 0 in practice), [1] poses whose
 * hull walk reached 200 edges, [2] poses over capacity, [3] faces whose first vertex had no
 * neighbour on its second plane. */
fxe_status fxe_last_stats(fxe_context* ctx, int32_t* out4);

/* Thermodynamics of an ensemble of n energies (kcal/mol) with multiplicities (NULL = all 1)
 * at temperature T (K), reduced on the device in FP64: StatMechEngine::compute. The arrays
 * are host memory. */
fxe_status fxe_thermo_compute(const double* energies, const int32_t* multiplicity, int64_t n,
                              double temperature, fxe_thermo* out);

/* Device-resident form of fxe_thermo_compute: d_energies / d_multiplicity are device
 * pointers; the reduction runs on `stream` (cudaStream_t or NULL) and is waited for. */
fxe_status fxe_thermo_compute_device(const double* d_energies, const int32_t* d_multiplicity,
                                     int64_t n, double temperature, fxe_thermo* out, void* stream);

/* Device-resident thermodynamics that allocates nothing. No reference counterpart.
 *
 * Same reduction as fxe_thermo_compute_device, for callers that must not allocate device
 * memory: code running under a fixed device-memory budget that has handed all free memory to
 * its own pools (an admission-controlled serving loop), and code that may not synchronise the
 * device, which every cudaMalloc/cudaFree can do. The block partials live in a fixed array
 * inside the library (FXE_THERMO_FIXED_MAX_BLOCKS partials of 32 bytes and one slot for a
 * counter, 2 MiB, one array per device), the merge runs on the device, and the record is written
 * to d_out (device memory).
 * Work is queued on `stream` (cudaStream_t or NULL for the legacy default stream) and not
 * waited for.
 *
 * - n may be at most FXE_THERMO_FIXED_MAX_N (FXE_THERMO_FIXED_MAX_BLOCKS partials, each of at most
 *   FXE_THERMO_FIXED_PER_THREAD x 256 energies); larger n is rejected with FXE_ERR_INVALID_ARGS
 *   before any work is queued.
 * - The first call on a device looks up the array's address (cudaGetSymbolAddress, with that
 *   device current) and loads the library's device code; make that first call before any stream
 *   capture and before memory is handed out. The address is kept for the life of the process:
 *   after a cudaDeviceReset the library's device code is loaded anew and the kept address no
 *   longer names the array, so do not call this entry point on a device that was reset.
 * - Nothing needs to start at zero: every partial a call reads is written by that call.
 * - Calls on one device share the array: calls whose work overlaps (different streams, or
 *   host threads without ordering) race and give wrong results. Serialise them on one stream.
 * - d_multiplicity entries must be positive (not checked on the device). */
#define FXE_THERMO_FIXED_PER_THREAD 16
#define FXE_THERMO_FIXED_MAX_BLOCKS 65536
#define FXE_THERMO_FIXED_MAX_N ((int64_t)FXE_THERMO_FIXED_MAX_BLOCKS * 256 * FXE_THERMO_FIXED_PER_THREAD)
fxe_status fxe_thermo_compute_device_fixed(const double* d_energies, const int32_t* d_multiplicity,
                                           int64_t n, double temperature, fxe_thermo* d_out,
                                           void* stream);

/* Boltzmann weights p_i = n_i exp(-beta E_i) / Z of the same ensemble
 * (StatMechEngine::boltzmann_weights, LIB/statmech.cpp:178-201). */
fxe_status fxe_thermo_weights(const double* energies, const int32_t* multiplicity, int64_t n,
                              double temperature, double* weights);

/* CF-based clustering of a docking result: cluster (LIB/cluster.cpp:9-182), the reference's
 * default clustering of the GA's ensemble (LIB/top.cpp:1351-1354; its file outputs come from
 * these results, see the Python writers).
 *
 * Input: n chromosomes as decoded ICs (n * n_genes, each within its gene limits, as the GA's
 * ensemble holds them: best first) and their apparent energies (app_evalue). The ligand of each
 * is built as calc_rmsd_chrom builds it (LIB/calc_rmsd_chrom.cpp:7-145). While chromosomes are
 * left and fewer than max_results (FA->max_results, default 10) clusters exist, the first
 * chromosome no cluster holds heads a new cluster, which takes in every later chromosome not yet
 * clustered whose ligand RMSD to the head (single precision over the ligand atoms in order) is
 * at most rmsd_threshold (FA->cluster_rmsd, default 2.0).
 * temperature (FA->temperature, K, an integer; 0, the reference's default, turns it off): with
 * beta = 1 / temperature (FA->beta as read_input sets it) and Z the sum of exp(-beta E) over all
 * n, a cluster's TCF is P E - T P ln P of its head and its ACF that plus P E + T P ln P of each
 * member (P = exp(-beta E) / Z), and the first min(max_results, n) entries are then reordered by
 * ACF with the reference's quicksort (QuickSort_Clusters); at temperature 0 the TCF is the
 * head's energy and the ACF the sum of the energies in the cluster.
 *
 * Outputs (host arrays, caller-owned): top, freq, tcf, acf [max_results]: the cluster entries in
 * the reference's final order (head chromosome, members counting the head, TCF, ACF; entries
 * past *n_clusters hold zeros, which the ACF sort can move forward, as in the reference);
 * member_of [n] (or NULL): the head of each chromosome's cluster, -1 for chromosomes left
 * unclustered after max_results clusters (the reference's Clus_GAPOP before its sort, which
 * also swaps the first entries of that per-chromosome array); rmsd [n] (or NULL): the RMSD of
 * each clustered chromosome to its head; top_rmsd [max_results^2] (or NULL): the RMSD between
 * the heads of entries a and b (row a), as calc_rmsd_chrom computes it for the .cad file.
 * FXE_ERR_INVALID_ARGS when an IC lies outside its gene limits or Z is zero (the reference stops
 * there, LIB/cluster.cpp:83-88). */
#define FXE_CLUSTER_MAX_N ((int64_t)1 << 30)
#define FXE_CLUSTER_MAX_RESULTS 1024
#define FXE_CLUSTER_MAX_GENES 100   /* the reference's MAX_NUM_GENES (LIB/gaboom.h:33) */
fxe_status fxe_cluster(fxe_context* ctx, int64_t n, const double* ic, const double* app_evalue,
                       int32_t temperature, float rmsd_threshold, int32_t max_results, int32_t* top,
                       int32_t* freq, double* tcf, double* acf, int32_t* member_of, float* rmsd,
                       float* top_rmsd, int32_t* n_clusters);

/* Device time (ms, CUDA events on the context's stream) of the kernels of the last fxe_cluster
 * call. No reference counterpart. */
fxe_status fxe_last_cluster_time(fxe_context* ctx, double* device_ms);

/* Per-stage device time of the evaluation calls. When enabled, every batch records CUDA events
 * around its three kernels (pose build, contact candidates, polyhedra and scoring) on the
 * batch's stream and waits for the last one, so fxe_eval_genes_device returns only after its
 * work is done. No reference counterpart (the reference times nothing below gaboom's
 * generation loop). */
fxe_status fxe_context_enable_timing(fxe_context* ctx, int32_t on);

/* Milliseconds per stage accumulated since the previous call (ms3[0] build, [1] contact
 * candidates, [2] polyhedra and scoring), and the number of kernels launched (counted whether
 * or not timing is enabled); resets both. */
fxe_status fxe_context_take_timing(fxe_context* ctx, double* ms3, int64_t* launches);

void fxe_context_destroy(fxe_context* ctx);

/* Batched evaluation: the populations of several contexts (different ligands, receptors, sizes)
 * scored by one launch of each kernel over all their poses, in place of one launch sequence per
 * population (the reference scores one population per cuda_eval_batch call). Each job names a
 * context, its chromosome count, its int32 genes and its output records; a context may appear
 * once per batch (its workspace holds that job's poses), all contexts share the batch's device
 * and one precision, and each job's n is at most its context's max_poses. Results equal those
 * of fxe_eval_genes on each context alone. */
typedef struct fxe_batch fxe_batch;
typedef struct fxe_job {
    fxe_context* ctx;
    int32_t n;
    const int32_t* genes;   /* n * n_genes of ctx */
    fxe_cf* out;            /* n records */
} fxe_job;

/* max_jobs jobs per call, max_poses poses in all, max_genes genes per chromosome (for staging
 * host chromosomes). */
fxe_status fxe_batch_create(int32_t max_jobs, int64_t max_poses, int32_t max_genes, fxe_batch** out);

/* Host genes and records; synchronous. */
fxe_status fxe_batch_eval_genes(fxe_batch* batch, const fxe_job* jobs, int32_t n_jobs);

/* Device genes and records; queued on `stream` (cudaStream_t, NULL: the batch's own stream) and
 * not waited for. A later call waits until this call's job table has been copied. */
fxe_status fxe_batch_eval_genes_device(fxe_batch* batch, const fxe_job* jobs, int32_t n_jobs, void* stream);

/* Kernels launched by the batch since the previous call (resets the count). */
fxe_status fxe_batch_take_launches(fxe_batch* batch, int64_t* launches);

void fxe_batch_destroy(fxe_batch* batch);

/* GA engine: docking jobs (one context each) run their genetic algorithm with the population in
 * HBM. A generation of every running job is one CUDA graph: breeding (roulette selection over
 * the job's fitness model, the reference's bit crossover and mutation, LIB/gaboom.cpp:909-960),
 * one batched evaluation of all children, BOOM or STEADY replacement (LIB/gaboom.cpp:1023-1033)
 * and the fitness of the new population (niche counts on the device). The graph is captured
 * again only when the set of running jobs changes, so jobs are admitted and retired between
 * generations (continuous batching).
 * Random draws are counter-based hashes of (seed, generation, child, draw): a job's trajectory
 * depends on its seed only, whatever else runs. Chromosomes the job has produced before are
 * dropped unless the job allows duplicates (fxe_ga_job.duplicates). */
typedef struct fxe_ga fxe_ga;
typedef struct fxe_ga_job {
    fxe_context* ctx;        /* the job's system; one running job per context */
    int32_t population;      /* 2..2048, at most ctx's max_poses */
    int32_t generations;
    double cross_rate;       /* probability of crossover per pair of children */
    double mut_rate;         /* probability of flipping each gene bit */
    uint64_t seed;
    int32_t n_new;           /* children per generation (0: population, BOOM's boom_fraction 1) */
    int32_t steady;          /* 1: STEADY replacement (n_new is steady_state_num), 0: BOOM */
    int32_t intragenes;      /* 1: crossover points inside genes, 0: at gene boundaries (default) */
    int32_t adaptive;        /* 1: adaptive probabilities from k[0..3] (adapt_prob) */
    double k[4];             /* k1..k4 (the reference's defaults: 1.0, 0.5, 1.0, 0.5) */
    int32_t duplicates;      /* 0 (the reference's default): a chromosome whose hash_genes
                                signature the job has produced before is dropped and another bred
                                (LIB/gaboom.cpp:977-1018, 1040-1045); 1: duplicates allowed */
    int32_t fitness;         /* FXE_FITNESS_PSHARE (0, the reference's default), _LINEAR, _SMFREE
                                (calculate_fitness, LIB/gaboom.cpp:1627-1760) */
    double sharing_alpha;    /* niche sharing: alpha, peaks, scale (0: the reference's defaults */
    double sharing_peaks;    /* 1, 5 and 10; sig_share as LIB/gaboom.cpp:300-309 forms it) */
    double sharing_scale;
    double entropy_weight;   /* SMFREE: weight of the Boltzmann term (the reference's default 0.5) */
    double temperature;      /* SMFREE: K (default 300); <= 0 ranks only, as the reference does */
} fxe_ga_job;

enum { FXE_FITNESS_PSHARE = 0, FXE_FITNESS_LINEAR = 1, FXE_FITNESS_SMFREE = 2 };

fxe_status fxe_ga_create(int32_t max_jobs, int32_t precision, fxe_ga** out);
/* Device bytes a job's GA state takes (populations, children, ensemble), for admission control. */
fxe_status fxe_ga_job_bytes(const fxe_ga_job* job, int64_t* bytes);
/* Draws, evaluates and sorts the job's initial population (waits for it); *slot names the job. */
fxe_status fxe_ga_admit(fxe_ga* ga, const fxe_ga_job* job, int32_t* slot);
/* One generation of every running job (queued; not waited for). */
fxe_status fxe_ga_step(fxe_ga* ga);
/* Waits for the queued generations and lists the slots whose jobs have finished. */
fxe_status fxe_ga_finished(fxe_ga* ga, int32_t* slots, int32_t cap, int32_t* n);
/* A finished job's best chromosome and energy, and the FP64 thermodynamics at `temperature` of
 * its ensemble as the reference assembles it (every generation's population, sorted by energy,
 * near-duplicates within 0.1 on every decoded gene removed, LIB/gaboom.cpp:494,520-540,
 * 2728-2747; StatMechEngine::compute, LIB/statmech.cpp:73-174), with the ensemble size in
 * *n_ensemble; frees the slot. The sort, the duplicate removal and the reduction run on the
 * device (the snapshots stay in HBM). */
fxe_status fxe_ga_collect(fxe_ga* ga, int32_t slot, double temperature, int32_t* best_genes,
                          double* best_energy, fxe_thermo* thermo, int64_t* n_ensemble);
/* A finished job's ensemble as fxe_ga_collect assembles it (best first, near-duplicates
 * removed): *n chromosomes as decoded ICs (n * n_genes, clamped as eval_chromosome leaves them)
 * and their energies, the input of fxe_cluster as the reference's cluster() receives
 * chrom_snapshot (LIB/top.cpp:1351-1354). With ic and energies NULL only *n is set; else cap
 * must be at least *n (FXE_ERR_CAPACITY otherwise). Call before fxe_ga_collect, which frees
 * the slot. */
fxe_status fxe_ga_ensemble(fxe_ga* ga, int32_t slot, int64_t cap, double* ic, double* energies,
                           int64_t* n);
/* The current population of a job (sorted by energy): P * n_genes genes and P energies. */
fxe_status fxe_ga_population(fxe_ga* ga, int32_t slot, int32_t* genes, double* energies);
/* Candidates a job has dropped as duplicates so far, and those taken although seen before
 * (when 16 batches of candidates in a row held too few new ones; 0 in practice). */
fxe_status fxe_ga_duplicates(fxe_ga* ga, int32_t slot, int64_t* rejected, int64_t* forced);
/* Kernels launched and graphs replayed since the previous call (resets both). */
fxe_status fxe_ga_take_launches(fxe_ga* ga, int64_t* launches, int64_t* graphs);
void fxe_ga_destroy(fxe_ga* ga);

/* genetoic (LIB/gaboom.cpp:2887-2906) of n chromosomes' int32 genes (n * n_genes, host memory) with
 * the context's gene limits, on the device: gene value g of gene q decodes to min + del * i for the
 * first bin i whose running total (set_bins' bin = 1 / nbin, LIB/gaboom.cpp:2295-2308, added in
 * order) reaches g / 2^31. clamp: 1 clamps into [min, max] as eval_chromosome does
 * (LIB/gaboom.cpp:1845-1866), 0 returns genetoic's value. Writes n * n_genes doubles to ic. No
 * separate reference entry point: the reference decodes inside its GA loop. */
fxe_status fxe_decode_genes(fxe_context* ctx, int64_t n, const int32_t* genes, int32_t clamp, double* ic);

/* One generation's breeding code of the GA engine run with the caller's draws in place of its
 * counter-based ones: for callers that drive the GA from their own random stream (the reference
 * draws from RandomDouble, LIB/gaboom.cpp:2942-2946) and for checking the operators alone.
 * Pair k: two roulette_wheel draws over `fitness` (LIB/gaboom.cpp:1158-1186), adapt_prob when
 * adaptive (:848-880, k4 = k1..k4), the crossover draw against the crossover probability, the
 * crossover's gene and bit-point draws (:2517-2614), then for each child and gene a rotamer draw
 * (rotamer genes only, :944-966) and 32 bit draws against the mutation probability (:2620-2641),
 * read in that order from draws[k * FXE_GA_DRAWS_PER_PAIR(n_genes) ...] (uniforms in [0, 1)).
 * pop: population * n_genes int32 genes; fitness: population values in roulette order; order: the
 * population index at each roulette position (NULL: 0, 1, ...); gene_prob: n_genes side-chain
 * probabilities of rotamer genes, -1 for the others (NULL: all -1). Outputs (host memory):
 * children 2 * n_pairs * n_genes (pair k's first child, then its second); draws_used[n_pairs] (or
 * NULL); fit_stats[3] (or NULL): fitness_stats' total, maximum and mean (LIB/gaboom.cpp:818-840).
 * Synchronous; allocates its device buffers per call. */
#define FXE_GA_DRAWS_PER_PAIR(ng) (7 + 2 * (int64_t)(ng) * 33)
fxe_status fxe_ga_breed_draws(int32_t population, int32_t n_genes, const int32_t* pop, const double* fitness,
                              const int32_t* order, const float* gene_prob, double cross_rate, double mut_rate,
                              int32_t intragenes, int32_t adaptive, const double* k4, int32_t n_pairs,
                              const double* draws, int32_t* children, int32_t* draws_used, double* fit_stats);

/* PSHARE's niche counts (LIB/gaboom.cpp:1652-1661) of a population given as ICs
 * (population * n_genes, host memory; population at most 2048): for each chromosome the sum over
 * all chromosomes, in order, of 1 - (rmsp / sig_share)^alpha for every calc_rmsp
 * (LIB/gaboom.cpp:2874-2885) within sig_share, computed by the GA engine's kernel. Writes
 * population doubles to share. */
fxe_status fxe_ga_niche_counts(int32_t population, int32_t n_genes, const double* ic, double sig_share,
                               double alpha, double* share);

/* The ensemble the reference's GA hands to statmech, assembled on the device from chromosomes given
 * as ICs: sorted by energy (QuickSort of chrom_snapshot, LIB/gaboom.cpp:520; equal energies keep
 * their input order, NaN sorts last), then remove_dups (LIB/gaboom.cpp:2728-2747): a chromosome is
 * dropped when every gene lies within 0.1 of the last chromosome kept. ic: n * n_genes, energies:
 * n (host memory, n < 2^31). Outputs (host memory, caller-owned, n entries suffice):
 * kept_index, kept_energy (either may be NULL): the input index and energy of each kept
 * chromosome in energy order; *n_kept their count. fxe_ga_collect and fxe_ga_ensemble run the
 * same device code on a job's snapshots. Allocates its device buffers per call. */
fxe_status fxe_ensemble_dedup(int64_t n, int32_t n_genes, const double* ic, const double* energies,
                              int64_t* kept_index, double* kept_energy, int64_t* n_kept);

/* Autotuner of the polyhedron launch. The launch hands poses to as many warps as the SMs hold; how
 * many run at once on an SM (the occupancy cap) trades latency hiding against contention for the
 * SM's double-precision pipe and instruction cache, differently for different ligand sizes and
 * batch sizes. fxe_context_autotune times the launch over this context's batch (d_genes: n int32
 * chromosomes in device memory, n <= max_poses) at every cap from half the SM's capacity to all of
 * it, `reps` timed launches each after one warm-up, and records the fastest in a process-wide table
 * keyed by size class: precision x scored atoms per pose (<= 16, 32, 64, more) x poses per launch
 * (<= 128, 512, 2048, 16384, more). Every later launch of that class, by any context, batch or GA
 * engine (captured when its set of jobs changes), uses it. Results never depend on the cap.
 * It then times the contact-candidate launch in both forms of fxe_context_set_cell_staging, as
 * fxe_context_autotune_contacts does, and records the faster for the class.
 * Outputs: the cap chosen (blocks per SM), and its fastest launch time (ms). Synchronous. No
 * reference counterpart. */
fxe_status fxe_context_autotune(fxe_context* ctx, int32_t n, const int32_t* d_genes, int32_t reps,
                                int32_t* blocks_per_sm, double* ms_per_launch);
/* Times the contact-candidate launch over this context's batch (d_genes: n int32 chromosomes in
 * device memory, n <= max_poses) with the cell entries read in place and staged in shared memory,
 * `reps` timed launches each after one warm-up, and records the faster form in the table for the
 * size class. ms2 (may be null): the fastest launch times in place and staged (ms); staged (may be
 * null): 1 when the staged form was the faster. Synchronous. */
fxe_status fxe_context_autotune_contacts(fxe_context* ctx, int32_t n, const int32_t* d_genes, int32_t reps,
                                         double* ms2, int32_t* staged);
/* The same sweep, reporting every cap it timed: caps[i] (blocks per SM) and ms[i] (fastest launch
 * time) for i < *n_out (at most max_out entries; the SM's capacity is at most 32 blocks). Records
 * the fastest in the table like fxe_context_autotune. */
fxe_status fxe_context_autotune_sweep(fxe_context* ctx, int32_t n, const int32_t* d_genes, int32_t reps,
                                      int32_t* caps, double* ms, int32_t max_out, int32_t* n_out);
/* The cap the table holds for a size class (0: not tuned, as many blocks as fit). */
fxe_status fxe_autotune_lookup(int32_t precision, int32_t scored_atoms, int64_t poses, int32_t* blocks_per_sm);

/* Message describing the last error on the calling thread ("" if none). */
const char* fxe_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* FXE_H */
