// fxe_common.cuh — device-side layout shared by the evaluation kernels.
//
// Layout in HBM (one evaluation context, resident for the context's lifetime):
//   receptor atoms as float4 (x, y, z, radius) in Calc order, and a copy of its rigid atoms
//   sorted by cell of the receptor's steady cell grid (the 6.5 A grid index_protein builds once
//   the receptor atoms are indexed, LIB/Vcontacts.cpp:1570-1715) with CSR offsets per cell;
//   flexible side chains (rotamer coordinates, residue bonded matrices, Calc places);
//   ligand build tree, genes and decode tables; energy matrix; cleft-grid ICs as float4.
// Per batch of poses (workspace sized at context creation for max_poses):
//   mobile-atom (side-chain and ligand) coordinates, cells and processing ranks per pose;
//   candidate lists (Calc index, squared distance) and Voronoi results (area, flags) per
//   (pose, mobile atom, slot).
#pragma once

#include <cstdint>

#include "../../include/fxe.h"

namespace fxe {

constexpr float kRw = 1.4f;              // LIB/flexaid.h:88
constexpr double kPi = 3.141592;         // LIB/flexaid.h:86
constexpr float kKwall = 1.0e6f;         // LIB/flexaid.h:78
constexpr float kCell = 6.5f;            // LIB/Vcontacts.h:56
constexpr double kClashThreshold = 1e4;  // LIB/flexaid.h:70
constexpr float kPolyPenalty = 1e6f;     // LIB/flexaid.h:69

// Per-atom workspace capacities of the Voronoi warp. Poses whose atoms exceed them are
// reported with FXE_POSE_CAPACITY rather than scored.
constexpr int kMaxCand = 96;    // contact candidates of one atom
constexpr int kMaxPlanes = kMaxCand + 4;
constexpr int kMaxEdges = 200;  // the reference aborts the hull walk at 200 edges
// vertex indices are bytes (255 means "none"); a walk that reaches the reference's 200-edge abort
// has at most about 135 vertices, a complete one with its arc points about 105
constexpr int kMaxVerts = 176;
constexpr int kMaxFacePts = 640;
constexpr int kMaxLig = 128;    // scored atoms per pose: ligand + side chains (bit masks, staging)
constexpr int kMaskWords = kMaxLig / 32;
constexpr int kMaxSc = 32;      // scored side-chain atoms per pose (one per lane)
constexpr int kMaxFlex = 8;     // flexible side chains

// candidate flag bits
constexpr uint8_t kOnHull = 1;    // plane flag != 'X'
constexpr uint8_t kEngulf = 2;    // plane flag 'E'
constexpr uint8_t kRecorded = 8;  // contact kept in the atom's record list

// atom status
constexpr int kAtomOk = 0;
constexpr int kAtomHullFail = 1;
constexpr int kAtomCapacity = 2;

struct DevSystem {
    // receptor
    int n_rec;
    const float4* rec_pos;       // [n_rec] x, y, z, radius (Calc order)
    const int* rec_type;         // [n_rec]
    float ori[3];
    float globalmin[3], globalmax[3], maxwidth;
    // steady cell grid of the receptor
    float gmin[3];
    float gmax[3];
    int dim;
    const int* cell_start;       // [dim^3 + 1]
    const int* cell_atom;        // [n_rec] Calc index, cell order
    const float4* cell_pos;      // [n_rec] positions in cell order
    // cleft grid
    int n_grid;
    const float4* grid_ic;       // dis, ang, dih, 0
    // ligand
    int n_lig;
    const float* lig_radius;
    const int* lig_type;
    const int4* lig_rec;         // rec[0..3], -1 = frame / no cascade
    const float* lig_shift;
    const float4* lig_ic;        // base dis, ang, dih
    int n_build;
    const int* build_order;
    // the rebuild list by dependency level: the atoms of one level have their build references in
    // earlier levels only, so a warp's lanes build them at once (n_levels 0: build in list order)
    int n_levels;
    const int* level_off;        // [n_levels + 1] into level_atom
    const int* level_atom;       // [n_build]
    const int8_t* bonded;        // [n_lig * n_lig]
    int n_genes;
    const int* gene_type;
    const int* gene_atom;
    const double* gene_min;
    const double* gene_max;
    const double* gene_del;
    const float* gene_minf;      // gene_min and 1 / gene_del in single precision (bin guesses)
    const float* gene_idelf;
    const int* dec_off;          // [n_genes + 1] offsets into dec_tab
    const double* dec_tab;       // running bin totals per gene
    // cosf/sinf of the host's C library for every single-precision angle the pose build can
    // meet, as (angle, cos, sin, the angle in degrees): per grid point (the anchor atom's angle and dihedral), and
    // per (ligand atom, angle|dihedral) over the bins of the gene that sets it last (trig_src:
    // -1 no gene, -2 the grid gene, else the gene's index; trig_off/trig_cnt locate its entries)
    const float4* grid_trig_a;   // [n_grid]
    const float4* grid_trig_d;   // [n_grid]
    const float4* trig_tab;
    const int* trig_src;         // [n_lig * 2]
    const int* trig_off;         // [n_lig * 2]
    const int* trig_cnt;         // [n_lig * 2]
    // the same replay for the distances (dis_src: -1 base, -2 grid, else the gene), and for each
    // dihedral a gene's cascade sets, the atoms whose shifts follow the gene's value in it
    const int* dis_src;          // [n_lig]
    const int* cas_off;          // [n_lig + 1] into cas_atom
    const int* cas_atom;
    // flexible side chains. Their non-backbone atoms ("side-chain atoms") are scored: with the
    // ligand atoms they form the pose's mobile atoms, side-chain atoms first (Calc order), then
    // the ligand (mobile index n_sc + l). Mobile atoms are re-placed every pose; the other
    // receptor atoms, the backbone of flexible residues included, stay where they are.
    int n_sc;
    int n_flex;
    const int* sc_slot;          // [n_sc] Calc index
    const int* sc_res;           // [n_sc] residue (0..n_flex-1)
    const int* sc_local;         // [n_sc] index among the residue's atoms
    const int* rec_mob;          // [n_rec] mobile index of a side-chain atom, -1 for the others
    const int* rec_res;          // [n_rec] residue << 8 | index in it, for atoms of flexible residues, else -1
    const float4* sc_rot;        // per residue: [n_rot][its side-chain atoms] x, y, z, radius
    const int4* flex_info;       // [n_flex] (first sc_rot entry, first mobile index, side-chain atoms, atoms)
    const int* flex_gene;        // [n_flex] the residue's rotamer gene
    const int* flex_bond_off;    // [n_flex] offset of the residue's bonded matrix
    const int8_t* flex_bonded;
    // energy matrix
    int ntypes;
    const int* em_weight;
    const int* em_off;
    const float* em_x;
    const float* em_y;
    // scoring switches
    float permeability;
    float dee_clash;
    int intramolecular;
    float solventterm;
};

struct DevWork {
    int max_poses;
    double* ic;            // [P * n_genes]
    // per (pose, mobile atom): P * (n_sc + n_lig) entries
    float4* mob_pos;       // x, y, z, radius
    int* mob_cell;
    int* mob_rank;         // position among the mobile atoms in Calclist order
    int4* pose_grid;       // [P] (altered, dim, 0, 0)
    float4* pose_gmin;     // [P]
    int* cand_idx;         // [P * n_mob * kMaxCand]
    float* cand_d2;        // [P * n_mob * kMaxCand]
    double* cand_area;     // [P * n_mob * kMaxCand]
    uint8_t* cand_flag;    // [P * n_mob * kMaxCand]
    int* cand_n;           // [P * n_mob]
    double* clash_part;    // [P * n_mob]
    int* pose_seed;        // [P * kMaxLig * 3] polyhedron seeds left by earlier atoms
    uint32_t* pose_rec;    // [P * kMaxLig * kMaskWords] mobile partners each processed atom kept
    fxe_cf* out;           // [P]
    int* counters;         // [4]: unused, hull failures, capacity, no-partner faces
    int* pose_order;       // [P] poses in the order pose_kernel takes them (costliest first)
};

// One job of a batched launch: a context's system and workspace (W.out pointing at the job's
// own output records), the job's chromosomes, and where its poses sit in the launch.
// Mobile atoms: the side-chain atoms (0 .. n_sc-1, Calc order), then the ligand atoms.
__device__ __forceinline__ int n_mobile(const DevSystem& S) { return S.n_sc + S.n_lig; }

// Calc index -> mobile index, or -1 for a receptor atom that stays in place.
__device__ __forceinline__ int mobile_of(const DevSystem& S, int j) {
    return j >= S.n_rec ? S.n_sc + (j - S.n_rec) : (S.n_sc ? S.rec_mob[j] : -1);
}

// Mobile index -> Calc index.
__device__ __forceinline__ int slot_of(const DevSystem& S, int m) {
    return m < S.n_sc ? S.sc_slot[m] : S.n_rec + (m - S.n_sc);
}

// How mobile atom m and the atom at Calc index j relate through their residue: 0 other
// residues, 1 one residue and at most bloops bonds apart (residue.bonded >= 0), 2 one residue
// and further apart.
__device__ __forceinline__ int residue_pair(const DevSystem& S, int m, int j) {
    if (m >= S.n_sc) {
        if (j < S.n_rec) return 0;
        return S.bonded[(m - S.n_sc) * S.n_lig + (j - S.n_rec)] >= 0 ? 1 : 2;
    }
    if (j >= S.n_rec) return 0;
    const int rr = S.rec_res[j], r = S.sc_res[m];
    if (rr < 0 || (rr >> 8) != r) return 0;
    return S.flex_bonded[S.flex_bond_off[r] + S.sc_local[m] * S.flex_info[r].w + (rr & 255)] >= 0 ? 1 : 2;
}

struct Job {
    DevSystem S;
    DevWork W;
    const int32_t* genes;  // [n * S.n_genes]
    int pose0;             // first pose of the job in the launch
    int n;                 // poses of the job
    long long warp0;       // first (pose, mobile atom) item of the job in the contact launch
};

// Index of the job holding launch item `key` (a pose, or a (pose, atom) item when by_warp):
// the last job whose first item is at or before key.
__device__ __forceinline__ int find_job(const Job* jobs, int n_jobs, long long key, bool by_warp) {
    int lo = 0, hi = n_jobs;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        const long long first = by_warp ? jobs[mid].warp0 : (long long)jobs[mid].pose0;
        if (first <= key) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Copies a job descriptor into shared memory with the lanes of one warp.
__device__ __forceinline__ void copy_job(Job* dst, const Job* src, int lane) {
    static_assert(sizeof(Job) % 4 == 0, "Job is copied in 4-byte words");
    const int* s = reinterpret_cast<const int*>(src);
    int* d = reinterpret_cast<int*>(dst);
    for (int k = lane; k < (int)(sizeof(Job) / 4); k += 32) d[k] = s[k];
    __syncwarp();
}

// One job's GA state in HBM. The population is double-buffered: selection writes the next
// population into pop_next / pop_e_next and swaps the pointers here, in device memory, so a
// captured generation can be replayed without the host.
struct GaJob {
    int32_t* pop;            // [P * ng] current population, sorted by energy
    int32_t* pop_next;
    double* pop_e;           // [P]
    double* pop_e_next;
    int32_t* child;          // [P * ng] chromosomes evaluated this generation
    const fxe_cf* child_cf;  // [P] their records
    int32_t* snap;           // [G * P * ng] the population after each generation (the snapshot
    double* snap_e;          // [G * P]       the reference feeds to statmech, LIB/gaboom.cpp:494)
    int* gen;                // [8] device counters: generation (advanced by selection), first
                             // candidate batch, duplicates forced / rejected, signature 0 seen
    uint64_t seed;
    double cross_rate, mut_rate;
    double k[4];             // adaptive probabilities (adapt_prob, LIB/gaboom.cpp:848-880)
    int P, ng, G;
    int nnew;                // children per generation
    int steady;              // 1: STEADY replacement, 0: BOOM
    int intragenes;          // crossover points inside genes (1) or at gene boundaries (0)
    int adaptive;            // adaptive crossover and mutation probabilities
    // duplicate rejection (hash_genes, LIB/gaboom.cpp:977-1018, 1040-1045): candidates are bred
    // in parallel and accepted in the reference's order against the set of every signature seen
    int reject;              // 1: reject duplicates (the reference's default, duplicates = false)
    int ncand;               // candidate pairs bred per generation
    int32_t* cand;           // [2 * ncand * ng]
    uint64_t* cand_sig;      // [2 * ncand]
    uint64_t* seen;          // open-addressing set of signatures (0 = empty), hmask + 1 slots
    unsigned long long hmask;
    // genetoic tables of the job's context (signatures are taken on decoded ICs)
    const int* dec_off;
    const double* dec_tab;
    const double* gene_min;
    const double* gene_del;
    const double* gene_max;
    const float* gene_prob;  // [ng] a rotamer gene's side-chain probability (flxsc.prob), -1 otherwise
    // fitness (calculate_fitness, LIB/gaboom.cpp:1627-1760) and the order roulette walks the
    // population in: energy order, or fitness order after a generation under PSHARE
    int fitness;             // kFitPshare, kFitLinear, kFitSmfree
    double sig_share;        // GB->sig_share (LIB/gaboom.cpp:300-309)
    double share_alpha;      // GB->alpha
    double ent_w;            // GB->entropy_weight
    double beta;             // 1 / (kB T) of SMFREE's Boltzmann weights; <= 0: rank only
    double* pic;             // [P * ng] ICs of the population, clamped as eval_chromosome leaves them
    double* share;           // [P] niche counts
    double* fit;             // [P] fitness at each roulette position
    double* fcum;            // [P] running sums of fit
    int* ford;               // [P] population index at each roulette position
    double* fstat;           // [4] total, maximum and mean fitness (fitness_stats)
};

constexpr int kFitPshare = 0;
constexpr int kFitLinear = 1;
constexpr int kFitSmfree = 2;

// one block's share of the ensemble reduction: running max of the log-weights and the sums
// of exp(lw - m), E exp(lw - m), E^2 exp(lw - m)
struct LsePart {
    double m, s, e1, e2;
};

// Device buffers and parameters of one clustering call (fxe_cluster). nb = cluster_blocks(n)
// blocks run each pass; R = max_results.
struct ClusterWork {
    int n;
    const double* ic;        // [n * n_genes]
    const double* e;         // [n] app_evalue
    float* xyz;              // [3 * n_lig * n] ligand coordinates by coordinate, then chromosome
    int* status;             // [1] set when a grid gene is out of range
    int temperature;         // K; 0: no Boltzmann terms
    double beta;             // 1 / temperature (read_input's FA->beta)
    float thr;               // RMSD threshold
    float exit_sum;          // a sum of squares past which the RMSD is above thr
    int max_results;
    double* part_z;          // [nb]
    int* member;             // [n] head of the chromosome's cluster, -1 none
    float* rmsd;             // [n]
    int* next;               // [R + 1] head of each cluster (n: none)
    double* part_acf;        // [R * nb]
    int* part_cnt;           // [R * nb]
    int* top;                // [R]
    int* freq;               // [R]
    double* tcf;             // [R]
    double* acf;             // [R]
    float* head_rmsd;        // [R * R] (the first n_clusters^2 entries are written)
    double* z;               // [1] partition function
};

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace fxe
