// fxe_flexaid.h — the GB300 evaluator as the CUDA backend of FlexAID∆S's GA.
//
// Compiled inside the reference's build (its headers flexaid.h and gaboom.h on the include path),
// linked with libfxe.so. It replaces the calls calculate_fitness makes to the CUDA surrogate
// (GPUContextPool::acquire_cuda -> cuda_eval_init -> cuda_eval_batch -> unpack_gpu_results,
// LIB/gaboom.cpp:1359-1386) with the evaluation ic2cf performs (LIB/ic2cf.cpp:18-386), on the
// device:
//
//   fxe_flexaid_pack     the set-up state top.cpp leaves before GA() (FA, atoms, residue,
//                        cleftgrid) as the C ABI's descriptors (include/fxe.h);
//   FxeFlexaidBackend    a context created from them; evaluate() scores the chromosomes of a
//                        population that are not yet evaluated (status != 'n') from their to_ic
//                        genes, clamped as eval_chromosome clamps them (LIB/gaboom.cpp:1845-1866),
//                        and writes cf, evalue and app_evalue back (get_cf_evalue,
//                        get_apparent_cf_evalue, LIB/ic2cf.cpp:389-402).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "flexaid.h"
#include "gaboom.h"
#include "fxe.h"

// The descriptors and the arrays they point into.
struct FxeFlexaidPacked {
    // receptor atoms in Calc order (residues 1 .. res_cnt, rotamer 0), the ligand residue excluded
    std::vector<float> rec_xyz, rec_radius;
    std::vector<int32_t> rec_type;
    std::vector<int32_t> calc_of_atom;   // atoms[] index -> receptor index (-1: not a receptor atom)
    std::vector<float> grid_ic;          // num_grd * 3 (entry 0: the ligand's initial anchor)
    // flexible side chains (FA->flex_res), rotamer coordinates and bonded matrices
    std::vector<fxe_flex_residue> flex;
    std::vector<std::vector<int8_t>> flex_backbone, flex_bonded;
    std::vector<std::vector<float>> flex_xyz;
    // ligand (FA->resligand), atoms numbered from its first atom
    std::vector<float> lig_radius, lig_shift, lig_ic;
    std::vector<int32_t> lig_type, lig_rec, build_order;
    std::vector<int8_t> bonded;
    std::vector<int32_t> gene_type, gene_atom, gene_map;
    std::vector<double> gene_min, gene_max, gene_del;
    // energy matrix (FA->energy_matrix): weight, curve offsets, curve points
    std::vector<int32_t> em_weight, em_offset;
    std::vector<float> em_x, em_y;

    fxe_receptor_desc receptor{};
    fxe_ligand_desc ligand{};
    fxe_emat_desc emat{};
    fxe_params params{};
};

// Fills *out from the reference's state. Returns false, with the reason in *err, for a state the
// evaluator does not take: a ligand residue that is not the last residue, normal-mode genes
// (type 3), a build reference outside the ligand, more atoms or side chains than the limits of
// include/fxe.h.
bool fxe_flexaid_pack(const FA_Global* FA, const atom* atoms, const resid* residue, const gridpoint* cleftgrid,
                      FxeFlexaidPacked* out, std::string* err);

class FxeFlexaidBackend {
public:
    FxeFlexaidBackend() = default;
    FxeFlexaidBackend(const FxeFlexaidBackend&) = delete;
    FxeFlexaidBackend& operator=(const FxeFlexaidBackend&) = delete;
    ~FxeFlexaidBackend();

    // Packs the state and creates the evaluation context on the current CUDA device, with room
    // for max_pop chromosomes per call (the reference's MAX_NUM_CHROM).
    bool init(const FA_Global* FA, const atom* atoms, const resid* residue, const gridpoint* cleftgrid,
              int max_pop, std::string* err);

    // Scores the chromosomes of chrom[0 .. pop_size) whose status is not 'n', as
    // unpack_gpu_results expects them back: cf (the whole cfstr), evalue, app_evalue, status 'n'.
    // Returns the number scored, or -1 with *err set.
    int evaluate(const FA_Global* FA, chromosome* chrom, int pop_size, int num_genes, std::string* err);

    const FxeFlexaidPacked& packed() const { return packed_; }

private:
    fxe_context* ctx_ = nullptr;
    FxeFlexaidPacked packed_;
    std::vector<double> icv_;
    std::vector<int> which_;
    std::vector<fxe_cf> out_;
};
