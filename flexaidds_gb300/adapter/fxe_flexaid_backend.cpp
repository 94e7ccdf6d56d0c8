// fxe_flexaid_backend.cpp — the evaluation context behind calculate_fitness's CUDA branch.
#include "fxe_flexaid.h"

FxeFlexaidBackend::~FxeFlexaidBackend() {
    if (ctx_) fxe_context_destroy(ctx_);
}

bool FxeFlexaidBackend::init(const FA_Global* FA, const atom* atoms, const resid* residue, const gridpoint* cleftgrid,
                             int max_pop, std::string* err) {
    if (ctx_) {
        fxe_context_destroy(ctx_);
        ctx_ = nullptr;
    }
    if (!fxe_flexaid_pack(FA, atoms, residue, cleftgrid, &packed_, err)) return false;
    if (fxe_context_create(&packed_.receptor, &packed_.ligand, &packed_.emat, &packed_.params, max_pop, &ctx_) !=
        FXE_OK) {
        if (err) *err = fxe_last_error();
        ctx_ = nullptr;
        return false;
    }
    return true;
}

int FxeFlexaidBackend::evaluate(const FA_Global* FA, chromosome* chrom, int pop_size, int num_genes,
                                std::string* err) {
    if (!ctx_ || num_genes != packed_.ligand.n_genes) {
        if (err) *err = ctx_ ? "gene count differs from the context's" : "backend not initialised";
        return -1;
    }
    // the chromosomes not yet evaluated, their ICs clamped as eval_chromosome clamps them
    which_.clear();
    icv_.clear();
    for (int c = 0; c < pop_size; ++c) {
        if (chrom[c].status == 'n') continue;
        which_.push_back(c);
        for (int g = 0; g < num_genes; ++g) {
            double v = chrom[c].genes[g].to_ic;
            if (v > FA->max_opt_par[g]) v = FA->max_opt_par[g];
            else if (v < FA->min_opt_par[g]) v = FA->min_opt_par[g];
            icv_.push_back(v);
        }
    }
    const int n = (int)which_.size();
    if (n == 0) return 0;
    out_.resize(n);
    if (fxe_eval_ic(ctx_, n, icv_.data(), out_.data()) != FXE_OK) {
        if (err) *err = fxe_last_error();
        return -1;
    }
    for (int k = 0; k < n; ++k)
        if (out_[k].status == FXE_POSE_CAPACITY) {
            // no reference counterpart (its workspaces are larger): the pose cannot be scored here
            if (err) *err = "a pose exceeded the evaluator's per-atom capacity";
            return -1;
        }
    for (int k = 0; k < n; ++k) {
        chromosome& ch = chrom[which_[k]];
        const fxe_cf& o = out_[k];
        ch.cf.com = o.com;
        ch.cf.con = o.con;
        ch.cf.wal = o.wal;
        ch.cf.sas = o.sas;
        ch.cf.elec = o.elec;
        ch.cf.gist = o.gist;
        ch.cf.hbond = o.hbond;
        ch.cf.gist_desolv = o.gist_desolv;
        ch.cf.metal_coord = o.metal_coord;
        ch.cf.totsas = o.totsas;
        ch.cf.rclash = o.rclash;
        ch.evalue = get_cf_evalue(&ch.cf);
        ch.app_evalue = get_apparent_cf_evalue(&ch.cf);
        ch.status = 'n';
    }
    return n;
}
