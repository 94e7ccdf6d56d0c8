// fxe_capi.cu — host side of the C ABI declared in include/fxe.h.
//
// A context owns the device copies of one receptor (with its cell list), one ligand (build
// tree, genes, decode tables) and one energy matrix, a workspace for max_poses poses and one
// CUDA stream. Batches larger than max_poses are scored in chunks.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "fxe_common.cuh"

namespace fxe {
void launch_build(const DevSystem&, const DevWork&, int, const int32_t*, const double*, cudaStream_t);
void launch_contacts(const DevSystem&, const DevWork&, int, cudaStream_t, bool);
void launch_order_poses(const DevSystem&, const DevWork&, int, cudaStream_t, int, int);
namespace f32 {
void launch_poses(const DevSystem&, const DevWork&, int, int*, uint8_t*, size_t, int, cudaStream_t);
cudaError_t configure_voronoi();
size_t pose_hist_bytes();
int pose_max_blocks_per_sm();
int pose_warps_per_block();
int pose_tile_for(int, size_t, int);
int pose_launch_blocks(int, size_t, int);
}
namespace f64 {
void launch_poses(const DevSystem&, const DevWork&, int, int*, uint8_t*, size_t, int, cudaStream_t);
cudaError_t configure_voronoi();
size_t pose_hist_bytes();
int pose_max_blocks_per_sm();
int pose_warps_per_block();
int pose_tile_for(int, size_t, int);
int pose_launch_blocks(int, size_t, int);
}

// How the pose order of a polyhedron launch over n poses may be dealt: {full tiles that start
// together (0: none, the order stays sorted), poses per tile}; the order kernel deals when those
// tiles are all the launch has or its scored poses do not fill them (launch_order_poses). Only
// lockstep launches have tiles.
struct Deal {
    int deal, tile;
};
inline Deal order_deal(int precision, int n, size_t hist_bytes, int blocks_per_sm) {
    const bool fast = precision == FXE_PRECISION_FAST;
    const int tile = fast ? f32::pose_tile_for(n, hist_bytes, blocks_per_sm)
                          : f64::pose_tile_for(n, hist_bytes, blocks_per_sm);
    if (tile < 1) return {0, 0};
    const int blocks = fast ? f32::pose_launch_blocks(n, hist_bytes, blocks_per_sm)
                            : f64::pose_launch_blocks(n, hist_bytes, blocks_per_sm);
    return {std::min(n / tile, blocks), tile};
}
// Face history of a polyhedron launch, large enough for either precision's launch: the warps the
// device holds at once, kHistStride bytes each (configure_voronoi first).
inline size_t pose_hist_bytes() {
    const size_t a = f32::pose_hist_bytes(), b = f64::pose_hist_bytes();
    return a > b ? a : b;
}
int cluster_blocks(int);
size_t ensemble_scratch_bytes(long long, int);
size_t grid_scratch_bytes(long long, long long);
cudaError_t launch_cleft_grid(int, const float*, const long long*, const int*, const float*, long long, long long, void*,
                              float*, long long*, cudaStream_t);
void launch_cleft_ic(const float*, long long, const float*, float*, cudaStream_t);
size_t cell_scratch_bytes(int, long long);
cudaError_t launch_cell_list(const float4*, const int*, int, const float*, int, void*, int*, int*, float4*, int*,
                             cudaStream_t);
cudaError_t launch_ensemble(long long, int, const double*, const double*, const DevSystem*, const int32_t*, void*,
                            long long*, double*, double*, int*, cudaStream_t);
cudaError_t launch_cluster(const DevSystem&, const ClusterWork&, cudaStream_t);
int thermo_blocks(long, int);
void launch_thermo_partial(const double*, const int32_t*, long, double, LsePart*, int, cudaStream_t);
void launch_thermo_weights(const double*, const int32_t*, long, double, double, double*, int, cudaStream_t);
void thermo_finish(const LsePart*, int, double, fxe_thermo*);
}  // namespace fxe

namespace {

thread_local std::string g_err;

fxe_status fail(fxe_status s, const std::string& msg) {
    g_err = msg;
    return s;
}

fxe_status cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? FXE_ERR_ALLOC : FXE_ERR_LAUNCH,
                std::string(what) + ": " + cudaGetErrorString(e));
}

// Device buffers of one call, freed when the call returns.
struct CallBuffers {
    std::vector<void*> p;
    template <typename T>
    cudaError_t get(T** out, size_t count) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
        if (e == cudaSuccess) {
            p.push_back(q);
            *out = reinterpret_cast<T*>(q);
        }
        return e;
    }
    template <typename T>
    cudaError_t put(T** out, const T* src, size_t count) {
        cudaError_t e = get(out, count);
        if (e == cudaSuccess && count) e = cudaMemcpy(*out, src, count * sizeof(T), cudaMemcpyHostToDevice);
        return e;
    }
    ~CallBuffers() {
        for (void* q : p) cudaFree(q);
    }
};


}  // namespace

// Device allocations freed together; a receptor's block is shared by every context built on it.
// The autotuner's table: per size class, the polyhedron launch's occupancy cap (blocks per SM, 0 =
// as many as fit) and the form of the contact-candidate scan (staged: the rigid cell entries
// staged in shared memory by bulk copies, 0 = read in place), process-wide, so that every
// context, batch and GA engine of the class uses what fxe_context_autotune measured for it.
// Classes: precision x scored atoms per pose (<= 16, 32, 64, more) x poses per launch (<= 128,
// 512, 2048, 16384, more). Neither choice changes a result.
struct Tune {
    int blocks = 0;
    int staged = 0;
};
std::mutex g_tune_mu;
std::map<int, Tune> g_tune;

int size_class(int precision, int mobile, long long poses) {
    const int m = mobile <= 16 ? 0 : mobile <= 32 ? 1 : mobile <= 64 ? 2 : 3;
    const int p = poses <= 128 ? 0 : poses <= 512 ? 1 : poses <= 2048 ? 2 : poses <= 16384 ? 3 : 4;
    return precision * 100 + m * 10 + p;
}

int tuned_blocks(int precision, int mobile, long long poses) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const auto it = g_tune.find(size_class(precision, mobile, poses));
    return it == g_tune.end() ? 0 : it->second.blocks;
}

bool tuned_staged(int precision, int mobile, long long poses) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const auto it = g_tune.find(size_class(precision, mobile, poses));
    return it != g_tune.end() && it->second.staged != 0;
}

// The contact scan's form for a setting (FXE_CELLS_*) and the launch's size class.
bool resolve_staged(int mode, int precision, int mobile, long long poses) {
    if (mode == FXE_CELLS_STAGED) return true;
    if (mode == FXE_CELLS_IN_PLACE) return false;
    return tuned_staged(precision, mobile, poses);
}

struct DevBlock {
    std::vector<void*> ptrs;
    std::vector<float4> grid_ic;   // host copy of the cleft-grid ICs
    std::vector<int> flex_nrot;    // rotamers of each flexible side chain
    std::vector<float> flex_prob;  // their flxsc.prob (GA engine)
    ~DevBlock() {
        for (void* p : ptrs) cudaFree(p);
    }
};

struct fxe_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    fxe::DevSystem S{};
    fxe::DevWork W{};
    std::vector<void*> allocs;
    std::shared_ptr<DevBlock> receptor = std::make_shared<DevBlock>();
    int rec_type_max = 0;             // largest receptor atom type (checked against each matrix)
    // host copies of the gene limits and genetoic tables (decoding snapshots on the host)
    std::vector<double> h_gmin, h_gmax, h_gdel;
    const void* rec_key = nullptr;    // identity of the receptor block (contexts sharing it)
    int32_t* d_genes = nullptr;
    double* d_icin = nullptr;
    int last_n = 0;
    int counters[4] = {0, 0, 0, 0};
    int precision = FXE_PRECISION_REFERENCE;
    int face_order = FXE_FACE_ORDER_REFERENCE;
    int cell_staging = FXE_CELLS_AUTO;
    uint8_t* d_hist = nullptr;        // face history of the polyhedron launch
    size_t hist_bytes = 0;
    // per-stage timing (fxe_context_enable_timing) and the count of kernels launched
    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    double stage_ms[3] = {0.0, 0.0, 0.0};
    int64_t launches = 0;
    double cluster_ms = 0.0;          // device time of the last fxe_cluster call

    template <typename T>
    cudaError_t alloc(T** p, size_t count) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
        if (e == cudaSuccess) {
            allocs.push_back(q);
            *p = reinterpret_cast<T*>(q);
        }
        return e;
    }
    template <typename T>
    cudaError_t upload(const T** dst, const T* src, size_t count) {
        T* d = nullptr;
        cudaError_t e = alloc(&d, count);
        if (e != cudaSuccess) return e;
        if (count) e = cudaMemcpy(d, src, count * sizeof(T), cudaMemcpyHostToDevice);
        *dst = d;
        return e;
    }
    template <typename T>
    cudaError_t upload_receptor(const T** dst, const T* src, size_t count) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
        if (e != cudaSuccess) return e;
        receptor->ptrs.push_back(q);
        if (count) e = cudaMemcpy(q, src, count * sizeof(T), cudaMemcpyHostToDevice);
        *dst = reinterpret_cast<const T*>(q);
        return e;
    }
    ~fxe_context() {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        for (void* p : allocs) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
};

extern "C" const char* fxe_last_error(void) { return g_err.c_str(); }

#define FXE_TRY(expr, what)                      \
    do {                                         \
        cudaError_t _e = (expr);                 \
        if (_e != cudaSuccess) return cuda_fail(_e, what); \
    } while (0)

namespace {

// The single-precision angle buildcc takes the sine and cosine of (LIB/buildcc.cpp:80-100),
// formed as the pose build kernel forms it.
float build_angle(float deg) { return (float)(deg * fxe::kPi / 180.0f); }

fxe_status context_create(const fxe_receptor_desc* rec, const fxe_context* share,
                          const fxe_ligand_desc* lig, const fxe_emat_desc* em, const fxe_params* prm,
                          int32_t max_poses, fxe_context** out) {
    g_err.clear();
    if ((!rec && !share) || !lig || !em || !prm || !out || max_poses <= 0)
        return fail(FXE_ERR_INVALID_ARGS, "null argument or max_poses <= 0");
    *out = nullptr;
    if (rec && (rec->n_atoms <= 0 || !rec->xyz || !rec->radius || !rec->type || rec->n_grid <= 0 || !rec->grid_ic))
        return fail(FXE_ERR_INVALID_ARGS, "receptor descriptor incomplete");
    if (lig->n_atoms < 3 || lig->n_atoms > fxe::kMaxLig)
        return fail(FXE_ERR_INVALID_ARGS, "ligand must have 3.." + std::to_string(fxe::kMaxLig) + " atoms");
    if (!lig->radius || !lig->type || !lig->rec || !lig->shift || !lig->ic || !lig->build_order ||
        !lig->bonded || lig->n_build <= 0 || lig->n_build > lig->n_atoms)
        return fail(FXE_ERR_INVALID_ARGS, "ligand descriptor incomplete");
    if (lig->n_genes < 0 || lig->n_genes > 1024 || (lig->n_genes && (!lig->gene_type || !lig->gene_atom ||
        !lig->gene_min || !lig->gene_max || !lig->gene_del || !lig->gene_map)))
        return fail(FXE_ERR_INVALID_ARGS, "gene arrays incomplete");
    // flexible side chains: the receptor's own, or those of the receptor shared
    std::vector<int> flex_nrot;
    int n_sc = 0;
    if (rec) {
        if (rec->n_flex < 0 || rec->n_flex > fxe::kMaxFlex || (rec->n_flex && !rec->flex))
            return fail(FXE_ERR_INVALID_ARGS, "at most " + std::to_string(fxe::kMaxFlex) + " flexible side chains");
        int next = 0;
        for (int r = 0; r < rec->n_flex; ++r) {
            const fxe_flex_residue& f = rec->flex[r];
            if (f.first < next || f.n_atoms < 1 || f.n_atoms > 255 || f.first + f.n_atoms > rec->n_atoms ||
                f.n_rot < 2 || !f.backbone || !f.rot_xyz || !f.bonded || !(f.prob >= 0.0f && f.prob <= 1.0f))
                return fail(FXE_ERR_INVALID_ARGS, "flexible side chain " + std::to_string(r) +
                                                      ": atoms out of order or range, fewer than two rotamers, or prob outside [0, 1]");
            next = f.first + f.n_atoms;
            int ns = 0;
            for (int k = 0; k < f.n_atoms; ++k) ns += f.backbone[k] ? 0 : 1;
            if (ns == 0) return fail(FXE_ERR_INVALID_ARGS, "flexible side chain without side-chain atoms");
            for (int k = 0; k < f.n_atoms * 3; ++k)
                if (f.rot_xyz[k] != rec->xyz[(size_t)f.first * 3 + k])
                    return fail(FXE_ERR_INVALID_ARGS, "rotamer 0 must be the receptor's own coordinates");
            n_sc += ns;
            flex_nrot.push_back(f.n_rot);
        }
    } else {
        flex_nrot = share->receptor->flex_nrot;
        n_sc = share->S.n_sc;
    }
    if (n_sc > fxe::kMaxSc)
        return fail(FXE_ERR_INVALID_ARGS, "more than " + std::to_string(fxe::kMaxSc) + " side-chain atoms");
    if (n_sc + lig->n_atoms > fxe::kMaxLig)
        return fail(FXE_ERR_INVALID_ARGS, "side-chain and ligand atoms exceed " + std::to_string(fxe::kMaxLig));
    std::vector<int> flex_gene(flex_nrot.size(), -1);
    for (int g = 0; g < lig->n_genes; ++g) {
        const int t = lig->gene_type[g];
        if (t != -1 && t != 0 && t != 1 && t != 2 && t != 4)
            return fail(FXE_ERR_INVALID_ARGS, "gene type " + std::to_string(t) + " is not supported (grid, distance, angle, dihedral, rotamer only)");
        if (!(lig->gene_del[g] > 0.0) || !(lig->gene_max[g] >= lig->gene_min[g]))
            return fail(FXE_ERR_INVALID_ARGS, "gene limits invalid");
        if (t == 4) {
            const int r = lig->gene_atom[g];
            if (r < 0 || r >= (int)flex_nrot.size() || flex_gene[r] >= 0)
                return fail(FXE_ERR_INVALID_ARGS, "rotamer gene names no flexible side chain, or one twice");
            if (!(lig->gene_min[g] >= 0.0) || !(lig->gene_max[g] + 0.5 < (double)flex_nrot[r]))
                return fail(FXE_ERR_INVALID_ARGS, "rotamer gene limits outside the residue's rotamers");
            flex_gene[r] = g;
        } else if (lig->gene_atom[g] < 0 || lig->gene_atom[g] >= lig->n_atoms) {
            return fail(FXE_ERR_INVALID_ARGS, "gene atom out of range");
        }
    }
    for (size_t r = 0; r < flex_gene.size(); ++r)
        if (flex_gene[r] < 0) return fail(FXE_ERR_INVALID_ARGS, "flexible side chain without a rotamer gene");
    for (int i = 0; i < lig->n_build; ++i)
        if (lig->build_order[i] < 0 || lig->build_order[i] >= lig->n_atoms)
            return fail(FXE_ERR_INVALID_ARGS, "build order entry out of range");
    for (int i = 0; i < lig->n_atoms * 4; ++i)
        if (lig->rec[i] < -1 || lig->rec[i] >= lig->n_atoms)
            return fail(FXE_ERR_INVALID_ARGS, "ligand rec entry out of range");
    if (em->ntypes <= 0 || !em->weight || !em->offset || !em->y || !em->x)
        return fail(FXE_ERR_INVALID_ARGS, "energy matrix incomplete");
    const int T = em->ntypes;
    int rec_type_max = share ? share->rec_type_max : 0;
    if (rec)
        for (int i = 0; i < rec->n_atoms; ++i) {
            if (rec->type[i] < 1) return fail(FXE_ERR_INVALID_ARGS, "receptor atom type out of range");
            rec_type_max = rec->type[i] > rec_type_max ? rec->type[i] : rec_type_max;
        }
    if (rec_type_max > T) return fail(FXE_ERR_INVALID_ARGS, "receptor atom type out of range");
    for (int i = 0; i < lig->n_atoms; ++i)
        if (lig->type[i] < 1 || lig->type[i] > T) return fail(FXE_ERR_INVALID_ARGS, "ligand atom type out of range");
    for (int k = 0; k < T * T; ++k)
        if (em->offset[k + 1] <= em->offset[k]) return fail(FXE_ERR_INVALID_ARGS, "energy matrix entry without values");

    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
        return fail(FXE_ERR_NO_DEVICE, "no CUDA device");

    auto* ctx = new fxe_context();
    fxe_status st = [&]() -> fxe_status {
        FXE_TRY(cudaGetDevice(&ctx->device), "cudaGetDevice");
        if (share && share->device != ctx->device)
            return fail(FXE_ERR_INVALID_ARGS, "the receptor's context lives on another device");
        FXE_TRY(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        FXE_TRY(fxe::f32::configure_voronoi(), "cudaFuncSetAttribute");
        FXE_TRY(fxe::f64::configure_voronoi(), "cudaFuncSetAttribute");
        fxe::DevSystem& S = ctx->S;
        ctx->rec_type_max = rec_type_max;
        const int n = lig->n_atoms;
        if (share) {
            // the receptor cache: this context reads the receptor, its cell list and cleft grid
            // from the device arrays of `share` and keeps them alive
            ctx->receptor = share->receptor;
            ctx->rec_key = share->rec_key;
            S = share->S;
        } else {
        ctx->rec_key = ctx->receptor.get();
        const int N = rec->n_atoms;
        // receptor atoms
        std::vector<float4> pos(N);
        for (int i = 0; i < N; ++i) pos[i] = make_float4(rec->xyz[3 * i], rec->xyz[3 * i + 1], rec->xyz[3 * i + 2], rec->radius[i]);
        S.n_rec = N;
        FXE_TRY(ctx->upload_receptor(&S.rec_pos, pos.data(), N), "receptor upload");
        FXE_TRY(ctx->upload_receptor(&S.rec_type, rec->type, N), "receptor upload");
        for (int k = 0; k < 3; ++k) {
            S.ori[k] = rec->ori[k];
            S.globalmin[k] = rec->globalmin[k];
            S.globalmax[k] = rec->globalmax[k];
            // index_protein's starting bounds once the receptor is indexed (LIB/Vcontacts.cpp:1596-1599)
            S.gmin[k] = (float)((int)rec->globalmin[k] + 1.0);
            S.gmax[k] = (float)((int)rec->globalmax[k] + 1.0);
        }
        S.maxwidth = rec->maxwidth;
        S.dim = (int)(rec->maxwidth / fxe::kCell) + 1;
        if (S.dim < 3) return fail(FXE_ERR_INVALID_ARGS, "receptor narrower than three cells");
        // flexible side chains: side-chain atoms leave the steady cell list (they move with the
        // pose); their rotamers, residue bonded matrices and Calc places go to the device
        std::vector<int> rec_mob(N, -1), rec_res(N, -1), sc_slot, sc_res, sc_local, bond_off;
        std::vector<float4> sc_rot;
        std::vector<int4> finfo;
        std::vector<int8_t> fbonded;
        for (int r = 0; r < rec->n_flex; ++r) {
            const fxe_flex_residue& f = rec->flex[r];
            const int sc0 = (int)sc_slot.size();
            for (int k = 0; k < f.n_atoms; ++k) {
                rec_res[f.first + k] = (r << 8) | k;
                if (f.backbone[k]) continue;
                rec_mob[f.first + k] = (int)sc_slot.size();
                sc_slot.push_back(f.first + k);
                sc_res.push_back(r);
                sc_local.push_back(k);
            }
            const int nsr = (int)sc_slot.size() - sc0;
            finfo.push_back(make_int4((int)sc_rot.size(), sc0, nsr, f.n_atoms));
            for (int q = 0; q < f.n_rot; ++q)
                for (int k = 0; k < f.n_atoms; ++k) {
                    if (f.backbone[k]) continue;
                    const float* x = f.rot_xyz + ((size_t)q * f.n_atoms + k) * 3;
                    sc_rot.push_back(make_float4(x[0], x[1], x[2], rec->radius[f.first + k]));
                }
            bond_off.push_back((int)fbonded.size());
            fbonded.insert(fbonded.end(), f.bonded, f.bonded + (size_t)f.n_atoms * f.n_atoms);
        }
        S.n_flex = rec->n_flex;
        S.n_sc = (int)sc_slot.size();
        ctx->receptor->flex_nrot = flex_nrot;
        for (int r = 0; r < rec->n_flex; ++r) ctx->receptor->flex_prob.push_back(rec->flex[r].prob);
        if (S.n_flex) {
            FXE_TRY(ctx->upload_receptor(&S.sc_slot, sc_slot.data(), sc_slot.size()), "side-chain upload");
            FXE_TRY(ctx->upload_receptor(&S.sc_res, sc_res.data(), sc_res.size()), "side-chain upload");
            FXE_TRY(ctx->upload_receptor(&S.sc_local, sc_local.data(), sc_local.size()), "side-chain upload");
            FXE_TRY(ctx->upload_receptor(&S.rec_mob, rec_mob.data(), N), "side-chain upload");
            FXE_TRY(ctx->upload_receptor(&S.rec_res, rec_res.data(), N), "side-chain upload");
            FXE_TRY(ctx->upload_receptor(&S.sc_rot, sc_rot.data(), sc_rot.size()), "side-chain upload");
            FXE_TRY(ctx->upload_receptor(&S.flex_info, finfo.data(), finfo.size()), "side-chain upload");
            FXE_TRY(ctx->upload_receptor(&S.flex_bond_off, bond_off.data(), bond_off.size()), "side-chain upload");
            FXE_TRY(ctx->upload_receptor(&S.flex_bonded, fbonded.data(), fbonded.size()), "side-chain upload");
        }
        // the steady cell list of the rigid atoms, built on the device (fxe_prepare.cu)
        const int dim = S.dim;
        const long long dim3 = (long long)dim * dim * dim;
        const int n_rigid = N - S.n_sc;
        {
            int *d_catom = nullptr, *d_mob = nullptr;
            float4* d_cpos = nullptr;
            CallBuffers cb;
            unsigned char* scratch = nullptr;
            FXE_TRY(cb.get(&scratch, fxe::cell_scratch_bytes(N, dim3)), "cell list scratch");
            if (S.n_sc) FXE_TRY(cb.put(&d_mob, rec_mob.data(), (size_t)N), "cell list");
            void* q = nullptr;
            FXE_TRY(cudaMalloc(&q, (size_t)(n_rigid > 0 ? n_rigid : 1) * sizeof(int) + 16), "cell list");
            ctx->receptor->ptrs.push_back(q);
            d_catom = static_cast<int*>(q);
            FXE_TRY(cudaMalloc(&q, (size_t)(n_rigid > 0 ? n_rigid : 1) * sizeof(float4) + 16), "cell list");
            ctx->receptor->ptrs.push_back(q);
            d_cpos = static_cast<float4*>(q);
            FXE_TRY(cudaMalloc(&q, ((size_t)dim3 + 1) * sizeof(int) + 16), "cell list");
            ctx->receptor->ptrs.push_back(q);
            int* d_start_keep = static_cast<int*>(q);
            int bad = 0;
            FXE_TRY(fxe::launch_cell_list(S.rec_pos, d_mob, N, S.gmin, dim, scratch, d_start_keep, d_catom, d_cpos, &bad,
                                          ctx->stream), "cell list build");
            if (bad) return fail(FXE_ERR_INVALID_ARGS, "receptor atom outside its own cell grid");
            S.cell_start = d_start_keep;
            S.cell_atom = d_catom;
            S.cell_pos = d_cpos;
        }
        // cleft grid
        std::vector<float4> gic(rec->n_grid);
        for (int g = 0; g < rec->n_grid; ++g)
            gic[g] = make_float4(rec->grid_ic[3 * g], rec->grid_ic[3 * g + 1], rec->grid_ic[3 * g + 2], 0.0f);
        S.n_grid = rec->n_grid;
        FXE_TRY(ctx->upload_receptor(&S.grid_ic, gic.data(), rec->n_grid), "grid upload");
        // the C library's cosf/sinf of the anchor atom's angle and dihedral at every grid point
        std::vector<float4> ta(rec->n_grid), td(rec->n_grid);
        for (int g = 0; g < rec->n_grid; ++g) {
            const float a = build_angle(gic[g].y), d = build_angle(gic[g].z);
            ta[g] = make_float4(a, cosf(a), sinf(a), gic[g].y);
            td[g] = make_float4(d, cosf(d), sinf(d), gic[g].z);
        }
        FXE_TRY(ctx->upload_receptor(&S.grid_trig_a, ta.data(), rec->n_grid), "grid upload");
        FXE_TRY(ctx->upload_receptor(&S.grid_trig_d, td.data(), rec->n_grid), "grid upload");
        ctx->receptor->grid_ic = gic;
        }
        // ligand
        S.n_lig = n;
        std::vector<int4> lrec(n);
        std::vector<float4> lic(n);
        for (int l = 0; l < n; ++l) {
            lrec[l] = make_int4(lig->rec[4 * l], lig->rec[4 * l + 1], lig->rec[4 * l + 2], lig->rec[4 * l + 3]);
            lic[l] = make_float4(lig->ic[3 * l], lig->ic[3 * l + 1], lig->ic[3 * l + 2], 0.0f);
        }
        FXE_TRY(ctx->upload(&S.lig_radius, lig->radius, n), "ligand upload");
        FXE_TRY(ctx->upload(&S.lig_type, lig->type, n), "ligand upload");
        FXE_TRY(ctx->upload(&S.lig_rec, lrec.data(), n), "ligand upload");
        FXE_TRY(ctx->upload(&S.lig_shift, lig->shift, n), "ligand upload");
        FXE_TRY(ctx->upload(&S.lig_ic, lic.data(), n), "ligand upload");
        S.n_build = lig->n_build;
        FXE_TRY(ctx->upload(&S.build_order, lig->build_order, lig->n_build), "ligand upload");
        {
            // dependency levels of the rebuild list: an atom's level is one more than its latest
            // build reference's; references outside the list or later in it, or an atom listed
            // twice, keep the list order
            std::vector<int> at(n, -1), level(n, 0);
            bool ok = true;
            for (int i = 0; i < lig->n_build; ++i) {
                if (at[lig->build_order[i]] >= 0) ok = false;   // an atom listed twice: list order
                at[lig->build_order[i]] = i;
            }
            int top = 0;
            for (int i = 0; i < lig->n_build && ok; ++i) {
                const int l = lig->build_order[i];
                int lv = 0;
                for (int r = 0; r < 3; ++r) {
                    const int j = lig->rec[4 * l + r];
                    if (j < 0) continue;
                    if (at[j] < 0 || at[j] >= i) ok = false;
                    else lv = std::max(lv, level[j] + 1);
                }
                level[l] = lv;
                top = std::max(top, lv);
            }
            S.n_levels = 0;
            if (ok) {
                std::vector<int> off(top + 2, 0), atoms;
                for (int i = 0; i < lig->n_build; ++i) ++off[level[lig->build_order[i]] + 1];
                for (int v = 0; v <= top; ++v) off[v + 1] += off[v];
                atoms.resize(lig->n_build);
                std::vector<int> fill(off.begin(), off.end() - 1);
                for (int i = 0; i < lig->n_build; ++i) atoms[fill[level[lig->build_order[i]]]++] = lig->build_order[i];
                S.n_levels = top + 1;
                FXE_TRY(ctx->upload(&S.level_off, off.data(), off.size()), "ligand upload");
                FXE_TRY(ctx->upload(&S.level_atom, atoms.data(), atoms.size()), "ligand upload");
            }
        }
        FXE_TRY(ctx->upload(&S.bonded, lig->bonded, (size_t)n * n), "ligand upload");
        // genes and genetoic decode tables (running bin totals, LIB/gaboom.cpp:2295-2308, 2887-2906)
        const int ng = lig->n_genes;
        S.n_genes = ng;
        std::vector<int> doff(ng + 1, 0);
        std::vector<double> dtab;
        for (int g = 0; g < ng; ++g) {
            double nbin = (lig->gene_max[g] - lig->gene_min[g]) / lig->gene_del[g];
            if (nbin - (int)nbin > 0.0) nbin += 1.0;
            if (lig->gene_map[g]) nbin += 1.0;
            if (!(nbin >= 1.0) || nbin > 5e7) return fail(FXE_ERR_INVALID_ARGS, "gene bin count out of range");
            const double bin = 1.0 / nbin;
            double tot = bin;
            dtab.push_back(tot);
            while (tot < 1.0) {
                tot += bin;
                dtab.push_back(tot);
            }
            doff[g + 1] = (int)dtab.size();
        }
        if (dtab.empty()) dtab.push_back(1.0);
        ctx->h_gmin.assign(lig->gene_min, lig->gene_min + ng);
        ctx->h_gmax.assign(lig->gene_max, lig->gene_max + ng);
        ctx->h_gdel.assign(lig->gene_del, lig->gene_del + ng);
        {
            // which gene sets each atom's angle and dihedral last, and through which cascade
            // (the IC assignment of ic2cf, LIB/ic2cf.cpp:53-105, replayed symbolically)
            std::vector<int> src(2 * n, -1), pos(2 * n, 0), dsrc(n, -1);
            std::vector<std::vector<int>> chain(ng);
            for (int g = 0; g < ng; ++g) {
                const int atm = lig->gene_atom[g], t = lig->gene_type[g];
                if (t == -1) {
                    src[2 * atm] = src[2 * atm + 1] = -2;
                    dsrc[atm] = -2;
                } else if (t == 0) {
                    dsrc[atm] = g;
                } else if (t == 1) {
                    src[2 * atm] = g;
                    pos[2 * atm] = 0;
                } else if (t == 2) {
                    chain[g].push_back(atm);
                    src[2 * atm + 1] = g;
                    pos[2 * atm + 1] = 0;
                    int j = atm, cat = lig->rec[4 * atm + 3], guard = 0;
                    if (cat >= 0)
                        while (cat != atm && guard++ <= n) {
                            chain[g].push_back(cat);
                            src[2 * cat + 1] = g;
                            pos[2 * cat + 1] = (int)chain[g].size() - 1;
                            j = cat;
                            cat = lig->rec[4 * j + 3];
                        }
                }
            }
            std::vector<float4> tab;
            std::vector<int> off(2 * n), cnt(2 * n);
            for (int l = 0; l < n; ++l)
                for (int c = 0; c < 2; ++c) {
                    const int k = 2 * l + c, g = src[k];
                    off[k] = (int)tab.size();
                    if (g == -2) {
                        cnt[k] = 0;   // read from the grid tables
                        continue;
                    }
                    std::vector<float> vals;
                    if (g == -1) {
                        vals.push_back(c == 0 ? lig->ic[3 * l + 1] : lig->ic[3 * l + 2]);
                    } else {
                        const int nb = doff[g + 1] - doff[g];
                        for (int i = 0; i < nb; ++i) {
                            double v = lig->gene_min[g] + lig->gene_del[g] * (double)i;
                            if (v > lig->gene_max[g]) v = lig->gene_max[g];
                            else if (v < lig->gene_min[g]) v = lig->gene_min[g];
                            float f = (float)v;
                            for (int q = 1; q <= pos[k]; ++q) f = f + lig->shift[chain[g][q]];
                            vals.push_back(f);
                        }
                    }
                    cnt[k] = (int)vals.size();
                    for (float a : vals) {
                        const float x = build_angle(a);
                        tab.push_back(make_float4(x, cosf(x), sinf(x), a));
                    }
                }
            if (tab.empty()) tab.push_back(make_float4(0.0f, 1.0f, 0.0f, 0.0f));   // never matched: cnt is 0
            FXE_TRY(ctx->upload(&S.trig_tab, tab.data(), tab.size()), "trig upload");
            FXE_TRY(ctx->upload(&S.trig_src, src.data(), 2 * n), "trig upload");
            FXE_TRY(ctx->upload(&S.trig_off, off.data(), 2 * n), "trig upload");
            FXE_TRY(ctx->upload(&S.trig_cnt, cnt.data(), 2 * n), "trig upload");
            // for a build that forms each atom's ICs without replaying the assignment: the gene
            // (or grid, -2; base, -1) that sets each distance last, and per atom whose dihedral a
            // gene's cascade sets, the atoms whose shifts are added after the gene's value
            std::vector<int> coff(n + 1, 0), catoms;
            for (int l = 0; l < n; ++l) {
                const int g = src[2 * l + 1];
                if (g >= 0)
                    for (int q = 1; q <= pos[2 * l + 1]; ++q) catoms.push_back(chain[g][q]);
                coff[l + 1] = (int)catoms.size();
            }
            if (catoms.empty()) catoms.push_back(0);
            FXE_TRY(ctx->upload(&S.dis_src, dsrc.data(), n), "trig upload");
            FXE_TRY(ctx->upload(&S.cas_off, coff.data(), n + 1), "trig upload");
            FXE_TRY(ctx->upload(&S.cas_atom, catoms.data(), catoms.size()), "trig upload");
        }
        if (!flex_gene.empty()) FXE_TRY(ctx->upload(&S.flex_gene, flex_gene.data(), flex_gene.size()), "gene upload");
        FXE_TRY(ctx->upload(&S.gene_type, lig->gene_type, ng), "gene upload");
        FXE_TRY(ctx->upload(&S.gene_atom, lig->gene_atom, ng), "gene upload");
        FXE_TRY(ctx->upload(&S.gene_min, lig->gene_min, ng), "gene upload");
        FXE_TRY(ctx->upload(&S.gene_max, lig->gene_max, ng), "gene upload");
        FXE_TRY(ctx->upload(&S.gene_del, lig->gene_del, ng), "gene upload");
        {
            std::vector<float> fmin(ng), fidel(ng);
            for (int g = 0; g < ng; ++g) {
                fmin[g] = (float)lig->gene_min[g];
                fidel[g] = (float)(1.0 / lig->gene_del[g]);
            }
            FXE_TRY(ctx->upload(&S.gene_minf, fmin.data(), ng), "gene upload");
            FXE_TRY(ctx->upload(&S.gene_idelf, fidel.data(), ng), "gene upload");
        }
        FXE_TRY(ctx->upload(&S.dec_off, doff.data(), ng + 1), "gene upload");
        FXE_TRY(ctx->upload(&S.dec_tab, dtab.data(), dtab.size()), "gene upload");
        // energy matrix
        S.ntypes = T;
        const int npts = em->offset[T * T];
        FXE_TRY(ctx->upload(&S.em_weight, em->weight, (size_t)T * T), "emat upload");
        FXE_TRY(ctx->upload(&S.em_off, em->offset, (size_t)T * T + 1), "emat upload");
        FXE_TRY(ctx->upload(&S.em_x, em->x, npts), "emat upload");
        FXE_TRY(ctx->upload(&S.em_y, em->y, npts), "emat upload");
        S.permeability = prm->permeability;
        S.dee_clash = prm->dee_clash;
        S.intramolecular = prm->intramolecular;
        S.solventterm = prm->solventterm;
        // workspace
        fxe::DevWork& W = ctx->W;
        const size_t P = (size_t)max_poses, PL = P * (size_t)(S.n_sc + n), PLC = PL * fxe::kMaxCand;
        W.max_poses = max_poses;
        FXE_TRY(ctx->alloc(&W.ic, P * (ng > 0 ? ng : 1)), "workspace");
        FXE_TRY(ctx->alloc(&W.mob_pos, PL), "workspace");
        FXE_TRY(ctx->alloc(&W.mob_cell, PL), "workspace");
        FXE_TRY(ctx->alloc(&W.mob_rank, PL), "workspace");
        FXE_TRY(ctx->alloc(&W.pose_grid, P), "workspace");
        FXE_TRY(ctx->alloc(&W.pose_gmin, P), "workspace");
        FXE_TRY(ctx->alloc(&W.cand_idx, PLC), "workspace");
        FXE_TRY(ctx->alloc(&W.cand_d2, PLC), "workspace");
        FXE_TRY(ctx->alloc(&W.cand_area, PLC), "workspace");
        FXE_TRY(ctx->alloc(&W.cand_flag, PLC), "workspace");
        FXE_TRY(ctx->alloc(&W.cand_n, PL), "workspace");
        FXE_TRY(ctx->alloc(&W.clash_part, PL), "workspace");
        FXE_TRY(ctx->alloc(&W.pose_seed, P * fxe::kMaxLig * 3), "workspace");
        FXE_TRY(ctx->alloc(&W.pose_rec, P * fxe::kMaxLig * fxe::kMaskWords), "workspace");
        FXE_TRY(ctx->alloc(&W.out, P), "workspace");
        FXE_TRY(ctx->alloc(&W.counters, 8), "workspace");   // [4]: the pose queue of pose_kernel
        FXE_TRY(ctx->alloc(&W.pose_order, P), "workspace");
        FXE_TRY(ctx->alloc(&ctx->d_genes, P * (ng > 0 ? ng : 1)), "staging");
        FXE_TRY(ctx->alloc(&ctx->d_icin, P * (ng > 0 ? ng : 1)), "staging");
        ctx->hist_bytes = fxe::pose_hist_bytes();
        FXE_TRY(ctx->alloc(&ctx->d_hist, ctx->hist_bytes), "face history");
        FXE_TRY(cudaDeviceSynchronize(), "context set-up");
        return FXE_OK;
    }();
    if (st != FXE_OK) {
        delete ctx;
        return st;
    }
    *out = ctx;
    return FXE_OK;
}

}  // namespace

extern "C" fxe_status fxe_context_create(const fxe_receptor_desc* rec, const fxe_ligand_desc* lig,
                                         const fxe_emat_desc* em, const fxe_params* prm,
                                         int32_t max_poses, fxe_context** out) {
    if (!rec) {
        g_err = "null argument or max_poses <= 0";
        return FXE_ERR_INVALID_ARGS;
    }
    return context_create(rec, nullptr, lig, em, prm, max_poses, out);
}

extern "C" fxe_status fxe_context_create_shared(const fxe_context* receptor_of, const fxe_ligand_desc* lig,
                                                const fxe_emat_desc* em, const fxe_params* prm,
                                                int32_t max_poses, fxe_context** out) {
    if (!receptor_of) {
        g_err = "receptor_of is NULL";
        return FXE_ERR_INVALID_ARGS;
    }
    return context_create(nullptr, receptor_of, lig, em, prm, max_poses, out);
}

namespace {

fxe_status run_chunk(fxe_context* ctx, int nb, const int32_t* d_genes, const double* d_ic,
                     cudaStream_t s) {
    const bool t = ctx->timing;
    if (t) cudaEventRecord(ctx->ev[0], s);
    fxe::launch_build(ctx->S, ctx->W, nb, d_genes, d_ic, s);
    if (t) cudaEventRecord(ctx->ev[1], s);
    fxe::launch_contacts(ctx->S, ctx->W, nb, s,
                         resolve_staged(ctx->cell_staging, ctx->precision, ctx->S.n_sc + ctx->S.n_lig, nb));
    if (t) cudaEventRecord(ctx->ev[2], s);
    uint8_t* hist = ctx->face_order == FXE_FACE_ORDER_REFERENCE ? ctx->d_hist : nullptr;
    const int bpsm = tuned_blocks(ctx->precision, ctx->S.n_sc + ctx->S.n_lig, nb);
    const fxe::Deal dl = fxe::order_deal(ctx->precision, nb, hist ? ctx->hist_bytes : 0, bpsm);
    fxe::launch_order_poses(ctx->S, ctx->W, nb, s, dl.deal, dl.tile);
    if (ctx->precision == FXE_PRECISION_FAST)
        fxe::f32::launch_poses(ctx->S, ctx->W, nb, ctx->W.counters + 4, hist, ctx->hist_bytes, bpsm, s);
    else fxe::f64::launch_poses(ctx->S, ctx->W, nb, ctx->W.counters + 4, hist, ctx->hist_bytes, bpsm, s);
    if (t) cudaEventRecord(ctx->ev[3], s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    ctx->launches += 4;
    if (t) {
        FXE_TRY(cudaEventSynchronize(ctx->ev[3]), "timing");
        for (int k = 0; k < 3; ++k) {
            float ms = 0.0f;
            FXE_TRY(cudaEventElapsedTime(&ms, ctx->ev[k], ctx->ev[k + 1]), "timing");
            ctx->stage_ms[k] += ms;
        }
    }
    return FXE_OK;
}

fxe_status eval_host(fxe_context* ctx, int32_t n, const int32_t* genes, const double* ic, fxe_cf* out) {
    g_err.clear();
    if (!ctx || n < 0 || (n > 0 && (!out || (!genes && !ic)))) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    const int ng = ctx->S.n_genes;
    const int P = ctx->W.max_poses;
    cudaStream_t s = ctx->stream;
    FXE_TRY(cudaMemsetAsync(ctx->W.counters, 0, 4 * sizeof(int), s), "counters");
    for (int off = 0; off < n; off += P) {
        const int nb = n - off < P ? n - off : P;
        if (genes) {
            FXE_TRY(cudaMemcpyAsync(ctx->d_genes, genes + (size_t)off * ng, (size_t)nb * ng * sizeof(int32_t),
                                    cudaMemcpyHostToDevice, s), "genes to device");
        } else {
            FXE_TRY(cudaMemcpyAsync(ctx->d_icin, ic + (size_t)off * ng, (size_t)nb * ng * sizeof(double),
                                    cudaMemcpyHostToDevice, s), "ICs to device");
        }
        fxe_status st = run_chunk(ctx, nb, genes ? ctx->d_genes : nullptr, genes ? nullptr : ctx->d_icin, s);
        if (st != FXE_OK) return st;
        FXE_TRY(cudaMemcpyAsync(out + off, ctx->W.out, (size_t)nb * sizeof(fxe_cf), cudaMemcpyDeviceToHost, s),
                "results to host");
    }
    FXE_TRY(cudaMemcpyAsync(ctx->counters, ctx->W.counters, 4 * sizeof(int), cudaMemcpyDeviceToHost, s), "counters");
    FXE_TRY(cudaStreamSynchronize(s), "evaluation");
    ctx->last_n = n < P ? n : P;
    return FXE_OK;
}

}  // namespace

extern "C" fxe_status fxe_eval_genes(fxe_context* ctx, int32_t n, const int32_t* genes, fxe_cf* out) {
    if (n > 0 && !genes) return fail(FXE_ERR_INVALID_ARGS, "genes is NULL");
    return eval_host(ctx, n, genes, nullptr, out);
}

extern "C" fxe_status fxe_eval_ic(fxe_context* ctx, int32_t n, const double* ic, fxe_cf* out) {
    if (n > 0 && !ic) return fail(FXE_ERR_INVALID_ARGS, "ic is NULL");
    return eval_host(ctx, n, nullptr, ic, out);
}

extern "C" fxe_status fxe_eval_genes_device(fxe_context* ctx, int32_t n, const int32_t* d_genes,
                                            fxe_cf* d_out, void* stream) {
    g_err.clear();
    if (!ctx || n < 0 || (n > 0 && (!d_genes || !d_out))) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    if (n > ctx->W.max_poses) return fail(FXE_ERR_INVALID_ARGS, "n exceeds the context's max_poses");
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    if (n == 0) return FXE_OK;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    FXE_TRY(cudaMemsetAsync(ctx->W.counters, 0, 4 * sizeof(int), s), "counters");
    fxe_status st = run_chunk(ctx, n, d_genes, nullptr, s);
    if (st != FXE_OK) return st;
    FXE_TRY(cudaMemcpyAsync(d_out, ctx->W.out, (size_t)n * sizeof(fxe_cf), cudaMemcpyDeviceToDevice, s), "results");
    ctx->last_n = n;
    return FXE_OK;
}

extern "C" fxe_status fxe_context_enable_timing(fxe_context* ctx, int32_t on) {
    g_err.clear();
    if (!ctx) return fail(FXE_ERR_INVALID_ARGS, "ctx is NULL");
    if (on && !ctx->ev[0]) {
        for (auto& e : ctx->ev) FXE_TRY(cudaEventCreate(&e), "timing events");
    }
    ctx->timing = on != 0;
    return FXE_OK;
}

extern "C" fxe_status fxe_context_take_timing(fxe_context* ctx, double* ms3, int64_t* launches) {
    g_err.clear();
    if (!ctx) return fail(FXE_ERR_INVALID_ARGS, "ctx is NULL");
    for (int k = 0; k < 3; ++k) {
        if (ms3) ms3[k] = ctx->stage_ms[k];
        ctx->stage_ms[k] = 0.0;
    }
    if (launches) *launches = ctx->launches;
    ctx->launches = 0;
    return FXE_OK;
}

extern "C" fxe_status fxe_last_contacts(fxe_context* ctx, int32_t pose, int32_t atom, int32_t cap,
                                        int32_t* partner, float* area, int32_t* n_out) {
    g_err.clear();
    if (!ctx || !n_out || pose < 0 || pose >= ctx->last_n || atom < 0 || atom >= ctx->S.n_sc + ctx->S.n_lig || cap < 0)
        return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    const size_t lb = (size_t)pose * (ctx->S.n_sc + ctx->S.n_lig) + atom;
    int nc = 0;
    FXE_TRY(cudaMemcpy(&nc, ctx->W.cand_n + lb, sizeof(int), cudaMemcpyDeviceToHost), "contacts");
    *n_out = 0;
    if (nc <= 0) return FXE_OK;
    std::vector<int> idx(nc);
    std::vector<double> ar(nc);
    std::vector<uint8_t> fl(nc);
    const size_t cb = lb * fxe::kMaxCand;
    FXE_TRY(cudaMemcpy(idx.data(), ctx->W.cand_idx + cb, nc * sizeof(int), cudaMemcpyDeviceToHost), "contacts");
    FXE_TRY(cudaMemcpy(ar.data(), ctx->W.cand_area + cb, nc * sizeof(double), cudaMemcpyDeviceToHost), "contacts");
    FXE_TRY(cudaMemcpy(fl.data(), ctx->W.cand_flag + cb, nc, cudaMemcpyDeviceToHost), "contacts");
    int k = 0;
    for (int c = nc - 1; c >= 0; --c) {  // newest record first, as vcfunction walks them
        if (!(fl[c] & fxe::kRecorded)) continue;
        if (k < cap) {
            if (partner) partner[k] = idx[c];
            if (area) area[k] = (float)ar[c];
        }
        ++k;
    }
    *n_out = k;
    return FXE_OK;
}

extern "C" fxe_status fxe_last_ligand_xyz(fxe_context* ctx, int32_t pose, float* xyz) {
    g_err.clear();
    if (!ctx || !xyz || pose < 0 || pose >= ctx->last_n) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    const int n = ctx->S.n_lig;
    std::vector<float4> v(n);
    FXE_TRY(cudaMemcpy(v.data(), ctx->W.mob_pos + (size_t)pose * (ctx->S.n_sc + n) + ctx->S.n_sc, n * sizeof(float4),
                       cudaMemcpyDeviceToHost),
            "ligand coordinates");
    for (int l = 0; l < n; ++l) {
        xyz[3 * l] = v[l].x;
        xyz[3 * l + 1] = v[l].y;
        xyz[3 * l + 2] = v[l].z;
    }
    return FXE_OK;
}

extern "C" fxe_status fxe_last_stats(fxe_context* ctx, int32_t* out4) {
    if (!ctx || !out4) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    for (int i = 0; i < 4; ++i) out4[i] = ctx->counters[i];
    return FXE_OK;
}

extern "C" fxe_status fxe_context_set_precision(fxe_context* ctx, int32_t precision) {
    g_err.clear();
    if (!ctx || (precision != FXE_PRECISION_REFERENCE && precision != FXE_PRECISION_FAST))
        return fail(FXE_ERR_INVALID_ARGS, "invalid precision mode");
    ctx->precision = precision;
    return FXE_OK;
}

extern "C" fxe_status fxe_context_set_face_order(fxe_context* ctx, int32_t mode) {
    g_err.clear();
    if (!ctx || (mode != FXE_FACE_ORDER_REFERENCE && mode != FXE_FACE_ORDER_GEOMETRIC))
        return fail(FXE_ERR_INVALID_ARGS, "invalid face order mode");
    ctx->face_order = mode;
    return FXE_OK;
}

extern "C" fxe_status fxe_context_set_cell_staging(fxe_context* ctx, int32_t mode) {
    g_err.clear();
    if (!ctx || (mode != FXE_CELLS_AUTO && mode != FXE_CELLS_IN_PLACE && mode != FXE_CELLS_STAGED))
        return fail(FXE_ERR_INVALID_ARGS, "invalid cell staging mode");
    ctx->cell_staging = mode;
    return FXE_OK;
}

extern "C" void fxe_context_destroy(fxe_context* ctx) { delete ctx; }

namespace {

// Block partials of the reduction, one buffer per device (a call reduces on the current device).
// Calls hold the lock until their partials are back on the host.
struct ThermoScratch {
    fxe::LsePart* part = nullptr;
    int cap = 0;
};
std::mutex g_thermo_mu;
std::map<int, ThermoScratch> g_thermo;

fxe_status thermo_run(const double* d_e, const int32_t* d_m, long n, double T, fxe_thermo* out,
                      double* d_w, cudaStream_t s) {
    int dev = 0, sms = 0;
    FXE_TRY(cudaGetDevice(&dev), "cudaGetDevice");
    FXE_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
    const int nb = fxe::thermo_blocks(n, sms);
    std::lock_guard<std::mutex> lk(g_thermo_mu);
    ThermoScratch& sc = g_thermo[dev];
    if (sc.cap < nb) {
        if (sc.part) cudaFree(sc.part);
        sc.part = nullptr;
        sc.cap = 0;
        FXE_TRY(cudaMalloc(&sc.part, nb * sizeof(fxe::LsePart)), "thermo scratch");
        sc.cap = nb;
    }
    const double beta = 1.0 / (0.001987206 * T);
    fxe::launch_thermo_partial(d_e, d_m, n, beta, sc.part, nb, s);
    FXE_TRY(cudaGetLastError(), "thermo launch");
    std::vector<fxe::LsePart> part(nb);
    FXE_TRY(cudaMemcpyAsync(part.data(), sc.part, nb * sizeof(fxe::LsePart), cudaMemcpyDeviceToHost, s), "thermo");
    FXE_TRY(cudaStreamSynchronize(s), "thermo");
    fxe_thermo th;
    fxe::thermo_finish(part.data(), nb, T, &th);
    if (out) *out = th;
    if (d_w) {
        fxe::launch_thermo_weights(d_e, d_m, n, beta, th.log_Z, d_w, nb, s);
        FXE_TRY(cudaGetLastError(), "thermo weights launch");
    }
    return FXE_OK;
}

fxe_status thermo_host(const double* e, const int32_t* mult, int64_t n, double T, fxe_thermo* out, double* w) {
    g_err.clear();
    if (!e || n <= 0 || !(T > 0.0)) return fail(FXE_ERR_INVALID_ARGS, "empty ensemble or T <= 0");
    if (mult)
        for (int64_t i = 0; i < n; ++i)
            if (mult[i] <= 0) return fail(FXE_ERR_INVALID_ARGS, "multiplicities must be positive");
    int dc = 0;
    if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0) return fail(FXE_ERR_NO_DEVICE, "no CUDA device");
    double *d_e = nullptr, *d_w = nullptr;
    int32_t* d_m = nullptr;
    cudaStream_t s = nullptr;
    auto cleanup = [&]() {
        if (d_e) cudaFree(d_e);
        if (d_w) cudaFree(d_w);
        if (d_m) cudaFree(d_m);
        if (s) cudaStreamDestroy(s);
    };
    fxe_status st = [&]() -> fxe_status {
        FXE_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
        FXE_TRY(cudaMalloc(&d_e, n * sizeof(double)), "thermo input");
        FXE_TRY(cudaMemcpyAsync(d_e, e, n * sizeof(double), cudaMemcpyHostToDevice, s), "thermo input");
        if (mult) {
            FXE_TRY(cudaMalloc(&d_m, n * sizeof(int32_t)), "thermo input");
            FXE_TRY(cudaMemcpyAsync(d_m, mult, n * sizeof(int32_t), cudaMemcpyHostToDevice, s), "thermo input");
        }
        if (w) FXE_TRY(cudaMalloc(&d_w, n * sizeof(double)), "thermo output");
        fxe_status r = thermo_run(d_e, d_m, n, T, out, d_w, s);
        if (r != FXE_OK) return r;
        if (w) {
            FXE_TRY(cudaMemcpyAsync(w, d_w, n * sizeof(double), cudaMemcpyDeviceToHost, s), "thermo output");
            FXE_TRY(cudaStreamSynchronize(s), "thermo output");
        }
        return FXE_OK;
    }();
    cleanup();
    return st;
}

}  // namespace

extern "C" fxe_status fxe_thermo_compute(const double* energies, const int32_t* multiplicity, int64_t n,
                                         double temperature, fxe_thermo* out) {
    if (!out) return fail(FXE_ERR_INVALID_ARGS, "out is NULL");
    return thermo_host(energies, multiplicity, n, temperature, out, nullptr);
}

extern "C" fxe_status fxe_thermo_weights(const double* energies, const int32_t* multiplicity, int64_t n,
                                         double temperature, double* weights) {
    if (!weights) return fail(FXE_ERR_INVALID_ARGS, "weights is NULL");
    return thermo_host(energies, multiplicity, n, temperature, nullptr, weights);
}

extern "C" fxe_status fxe_thermo_compute_device(const double* d_energies, const int32_t* d_multiplicity,
                                                int64_t n, double temperature, fxe_thermo* out, void* stream) {
    g_err.clear();
    if (!d_energies || n <= 0 || !(temperature > 0.0) || !out)
        return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    return thermo_run(d_energies, d_multiplicity, n, temperature, out, nullptr, (cudaStream_t)stream);
}

// ------------------------------------------------------------------------------------------
// fxe_cluster: CF-based clustering of a docking result (LIB/cluster.cpp:9-182).
// ------------------------------------------------------------------------------------------
namespace {

// QuickSort_Clusters (LIB/cluster.cpp:323-363): the reference's quicksort of the cluster entries
// beg..end by ACF, ascending (QS_ASC, LIB/gaboom.h:40), with its pivots and swaps, so that equal
// ACFs end where the reference puts them. perm follows the entries (each one's index before the
// sort).
void quicksort_clusters(int* top, int* fre, double* tcf, double* acf, int* perm, int beg, int end) {
    auto swap_at = [&](int x, int y) {
        std::swap(top[x], top[y]);
        std::swap(fre[x], fre[y]);
        std::swap(tcf[x], tcf[y]);
        std::swap(acf[x], acf[y]);
        std::swap(perm[x], perm[y]);
    };
    while (beg < end) {
        int l = beg, p = beg + (end - beg) / 2, r = end;
        const double piv = acf[p];
        while (true) {
            while (l <= r && (acf[l] - piv) <= 0) ++l;
            while (l <= r && (acf[r] - piv) > 0) --r;
            if (l > r) break;
            swap_at(l, r);
            if (p == r) p = l;
            ++l;
            --r;
        }
        swap_at(p, r);
        --r;
        if ((r - beg) < (end - l)) {
            quicksort_clusters(top, fre, tcf, acf, perm, beg, r);
            beg = l;
        } else {
            quicksort_clusters(top, fre, tcf, acf, perm, l, end);
            end = r;
        }
    }
}

struct DevScratch {
    std::vector<void*> p;
    template <typename T>
    cudaError_t get(T** out, size_t count) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
        if (e == cudaSuccess) p.push_back(q);
        *out = reinterpret_cast<T*>(q);
        return e;
    }
    ~DevScratch() {
        for (void* q : p) cudaFree(q);
    }
};

}  // namespace

extern "C" fxe_status fxe_cluster(fxe_context* ctx, int64_t n, const double* ic, const double* app_evalue,
                                  int32_t temperature, float rmsd_threshold, int32_t max_results,
                                  int32_t* top, int32_t* freq, double* tcf, double* acf, int32_t* member_of,
                                  float* rmsd, float* top_rmsd, int32_t* n_clusters) {
    g_err.clear();
    if (!ctx || !ic || !app_evalue || !top || !freq || !tcf || !acf || !n_clusters)
        return fail(FXE_ERR_INVALID_ARGS, "NULL argument");
    if (n < 1 || n > FXE_CLUSTER_MAX_N) return fail(FXE_ERR_INVALID_ARGS, "n out of range");
    if (temperature < 0 || !(rmsd_threshold >= 0.0f) || max_results < 1 || max_results > FXE_CLUSTER_MAX_RESULTS)
        return fail(FXE_ERR_INVALID_ARGS, "temperature < 0, rmsd_threshold < 0 or max_results out of range");
    if (ctx->S.n_genes > FXE_CLUSTER_MAX_GENES)
        return fail(FXE_ERR_INVALID_ARGS, "clustering takes ligands of at most " +
                                              std::to_string(FXE_CLUSTER_MAX_GENES) + " genes");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    const int N = (int)n, R = max_results, ng = ctx->S.n_genes, nl = ctx->S.n_lig;
    const int nb = fxe::cluster_blocks(N);
    cudaStream_t st = ctx->stream;
    DevScratch m;
    fxe::ClusterWork C{};
    C.n = N;
    C.temperature = temperature;
    C.beta = temperature > 0 ? (double)(1.0 / temperature) : 0.0;   // read_input's FA->beta
    C.thr = rmsd_threshold;
    // a float sum above thr^2 * n_atoms * (1 + 1e-5) gives sqrtf(sum / n_atoms) > thr whatever
    // the rounding of the division and the root
    {
        const double lim = (double)rmsd_threshold * rmsd_threshold * nl * (1.0 + 1e-5);
        float f = (float)lim;
        if ((double)f < lim) f = std::nextafter(f, INFINITY);
        C.exit_sum = f;
    }
    C.max_results = R;
    double* d_ic = nullptr;
    double* d_e = nullptr;
    FXE_TRY(m.get(&d_ic, (size_t)N * ng), "cluster ICs");
    FXE_TRY(m.get(&d_e, (size_t)N), "cluster energies");
    C.ic = d_ic;
    C.e = d_e;
    FXE_TRY(m.get(&C.xyz, (size_t)3 * nl * N), "cluster coordinates");
    FXE_TRY(m.get(&C.status, 1), "cluster status");
    FXE_TRY(m.get(&C.part_z, (size_t)nb), "cluster partials");
    FXE_TRY(m.get(&C.member, (size_t)N), "cluster members");
    FXE_TRY(m.get(&C.rmsd, (size_t)N), "cluster rmsd");
    FXE_TRY(m.get(&C.next, (size_t)R + 1), "cluster heads");
    FXE_TRY(m.get(&C.part_acf, (size_t)R * nb), "cluster partials");
    FXE_TRY(m.get(&C.part_cnt, (size_t)R * nb), "cluster partials");
    FXE_TRY(m.get(&C.top, (size_t)R), "cluster results");
    FXE_TRY(m.get(&C.freq, (size_t)R), "cluster results");
    FXE_TRY(m.get(&C.tcf, (size_t)R), "cluster results");
    FXE_TRY(m.get(&C.acf, (size_t)R), "cluster results");
    FXE_TRY(m.get(&C.head_rmsd, (size_t)R * R), "cluster results");
    FXE_TRY(m.get(&C.z, 1), "cluster results");
    std::vector<int> h_next(R + 1, N);
    h_next[0] = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    FXE_TRY(cudaEventCreate(&ev[0]), "cluster events");
    if (cudaEventCreate(&ev[1]) != cudaSuccess) {
        cudaEventDestroy(ev[0]);
        return fail(FXE_ERR_LAUNCH, "cluster events");
    }
    struct EvGuard {
        cudaEvent_t* e;
        ~EvGuard() {
            cudaEventDestroy(e[0]);
            cudaEventDestroy(e[1]);
        }
    } ev_guard{ev};
    FXE_TRY(cudaMemcpyAsync(d_ic, ic, sizeof(double) * N * ng, cudaMemcpyHostToDevice, st), "cluster ICs");
    FXE_TRY(cudaMemcpyAsync(d_e, app_evalue, sizeof(double) * N, cudaMemcpyHostToDevice, st), "cluster energies");
    FXE_TRY(cudaMemcpyAsync(C.next, h_next.data(), sizeof(int) * (R + 1), cudaMemcpyHostToDevice, st), "cluster heads");
    FXE_TRY(cudaMemsetAsync(C.member, 0xff, sizeof(int) * N, st), "cluster members");
    FXE_TRY(cudaMemsetAsync(C.rmsd, 0, sizeof(float) * N, st), "cluster rmsd");
    FXE_TRY(cudaMemsetAsync(C.status, 0, sizeof(int), st), "cluster status");
    FXE_TRY(cudaEventRecord(ev[0], st), "cluster events");
    FXE_TRY(fxe::launch_cluster(ctx->S, C, st), "cluster launch");
    FXE_TRY(cudaEventRecord(ev[1], st), "cluster events");
    ctx->launches += 2 + (temperature > 0 ? 1 : 0) + R;
    std::vector<int> h_top(R), h_freq(R);
    std::vector<double> h_tcf(R), h_acf(R);
    std::vector<float> h_hr((size_t)R * R);
    int status = 0;
    double z = 0.0;
    FXE_TRY(cudaMemcpyAsync(h_next.data(), C.next, sizeof(int) * (R + 1), cudaMemcpyDeviceToHost, st), "cluster results");
    FXE_TRY(cudaMemcpyAsync(h_top.data(), C.top, sizeof(int) * R, cudaMemcpyDeviceToHost, st), "cluster results");
    FXE_TRY(cudaMemcpyAsync(h_freq.data(), C.freq, sizeof(int) * R, cudaMemcpyDeviceToHost, st), "cluster results");
    FXE_TRY(cudaMemcpyAsync(h_tcf.data(), C.tcf, sizeof(double) * R, cudaMemcpyDeviceToHost, st), "cluster results");
    FXE_TRY(cudaMemcpyAsync(h_acf.data(), C.acf, sizeof(double) * R, cudaMemcpyDeviceToHost, st), "cluster results");
    FXE_TRY(cudaMemcpyAsync(h_hr.data(), C.head_rmsd, sizeof(float) * R * R, cudaMemcpyDeviceToHost, st), "cluster results");
    FXE_TRY(cudaMemcpyAsync(&status, C.status, sizeof(int), cudaMemcpyDeviceToHost, st), "cluster results");
    FXE_TRY(cudaMemcpyAsync(&z, C.z, sizeof(double), cudaMemcpyDeviceToHost, st), "cluster results");
    if (member_of)
        FXE_TRY(cudaMemcpyAsync(member_of, C.member, sizeof(int) * N, cudaMemcpyDeviceToHost, st), "cluster members");
    if (rmsd) FXE_TRY(cudaMemcpyAsync(rmsd, C.rmsd, sizeof(float) * N, cudaMemcpyDeviceToHost, st), "cluster rmsd");
    FXE_TRY(cudaStreamSynchronize(st), "cluster");
    float ms = 0.0f;
    FXE_TRY(cudaEventElapsedTime(&ms, ev[0], ev[1]), "cluster events");
    ctx->cluster_ms = ms;
    if (status & 2) return fail(FXE_ERR_INVALID_ARGS, "an IC lies outside its gene limits");
    if (status & 1) return fail(FXE_ERR_INVALID_ARGS, "a grid gene names no cleft point");
    if (temperature > 0 && z == 0.0)
        return fail(FXE_ERR_INVALID_ARGS, "the partition function of the clustering step is zero");
    int nc = 0;
    while (nc < R && h_next[nc] < N) ++nc;
    std::vector<int> perm(R);
    for (int k = 0; k < R; ++k) perm[k] = k;
    // the reference sorts its first max_results entries (LIB/cluster.cpp:177-181); its arrays
    // hold num_chrom entries, so at most n of them here
    if (temperature > 0) quicksort_clusters(h_top.data(), h_freq.data(), h_tcf.data(), h_acf.data(), perm.data(), 0,
                                            (R < N ? R : N) - 1);
    for (int k = 0; k < R; ++k) {
        top[k] = h_top[k];
        freq[k] = h_freq[k];
        tcf[k] = h_tcf[k];
        acf[k] = h_acf[k];
    }
    if (top_rmsd)
        for (int a = 0; a < R; ++a)
            for (int b = 0; b < R; ++b) {
                // entries past the clusters formed name chromosome 0, the first cluster's head
                const int ca = perm[a] < nc ? perm[a] : 0, cb = perm[b] < nc ? perm[b] : 0;
                top_rmsd[(size_t)a * R + b] = h_hr[(size_t)ca * nc + cb];
            }
    *n_clusters = nc;
    return FXE_OK;
}

extern "C" fxe_status fxe_last_cluster_time(fxe_context* ctx, double* device_ms) {
    g_err.clear();
    if (!ctx || !device_ms) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    *device_ms = ctx->cluster_ms;
    return FXE_OK;
}

// ------------------------------------------------------------------------------------------
// fxe_thermo_compute_device_fixed: the reduction with library-owned scratch, no allocation.
// ------------------------------------------------------------------------------------------
namespace fxe {
cudaError_t fixed_scratch_address(LsePart** p);
void launch_thermo_fixed(const double*, const int32_t*, long, double, double, LsePart*, fxe_thermo*,
                         cudaStream_t);
}  // namespace fxe

namespace {
constexpr int kFixedMaxDevices = 64;
std::atomic<fxe::LsePart*> g_fixed_scratch[kFixedMaxDevices];
}  // namespace

extern "C" fxe_status fxe_thermo_compute_device_fixed(const double* d_energies, const int32_t* d_multiplicity,
                                                      int64_t n, double temperature, fxe_thermo* d_out,
                                                      void* stream) {
    g_err.clear();
    if (!d_energies || !d_out || n <= 0 || !(temperature > 0.0))
        return fail(FXE_ERR_INVALID_ARGS, "invalid arguments (NULL pointer, n <= 0 or T <= 0)");
    if (n > FXE_THERMO_FIXED_MAX_N)
        return fail(FXE_ERR_INVALID_ARGS, "n = " + std::to_string(n) + " exceeds FXE_THERMO_FIXED_MAX_N = " +
                                              std::to_string((long long)FXE_THERMO_FIXED_MAX_N) +
                                              " (the fixed scratch holds " +
                                              std::to_string(FXE_THERMO_FIXED_MAX_BLOCKS) + " block partials)");
    int dev = 0;
    FXE_TRY(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kFixedMaxDevices) return fail(FXE_ERR_NO_DEVICE, "device ordinal out of range");
    fxe::LsePart* scratch = g_fixed_scratch[dev].load(std::memory_order_acquire);
    if (!scratch) {
        // set-up, once per device, with that device current
        FXE_TRY(fxe::fixed_scratch_address(&scratch), "cudaGetSymbolAddress of the fixed scratch");
        g_fixed_scratch[dev].store(scratch, std::memory_order_release);
    }
    const double beta = 1.0 / (0.001987206 * temperature);  // LIB/statmech.h:26
    fxe::launch_thermo_fixed(d_energies, d_multiplicity, (long)n, beta, temperature, scratch, d_out,
                             (cudaStream_t)stream);
    FXE_TRY(cudaGetLastError(), "fixed-scratch thermo launch");
    return FXE_OK;
}

// ------------------------------------------------------------------------------------------
// Batched evaluation: the populations of several contexts in one launch of each kernel.
// ------------------------------------------------------------------------------------------
namespace fxe {
void launch_build_jobs(const Job*, int, int, cudaStream_t);
void launch_contacts_jobs(const Job*, int, long long, cudaStream_t, bool);
void launch_order_poses_jobs(const Job*, int, int, int*, cudaStream_t, int, int);
namespace f32 {
void launch_poses_jobs(const Job*, int, int, int*, const int*, uint8_t*, size_t, int, cudaStream_t);
}
namespace f64 {
void launch_poses_jobs(const Job*, int, int, int*, const int*, uint8_t*, size_t, int, cudaStream_t);
}
}  // namespace fxe

struct fxe_batch {
    int device = 0;
    int max_jobs = 0;
    int64_t max_poses = 0;
    int32_t max_genes = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t staged = nullptr;          // the job table's host staging may be rewritten
    fxe::Job* d_jobs = nullptr;
    fxe::Job* h_jobs = nullptr;            // pinned
    int32_t* d_genes = nullptr;            // host-pointer form: staged chromosomes
    int32_t* h_genes = nullptr;            // pinned
    fxe_cf* d_out = nullptr;
    fxe_cf* h_out = nullptr;               // pinned
    int* d_next = nullptr;                 // pose queue of the polyhedron launch
    int* d_order = nullptr;                // [max_poses] its order (order_poses_jobs_kernel)
    uint8_t* d_hist = nullptr;             // face history of the polyhedron launch
    size_t hist_bytes = 0;
    int64_t launches = 0;
    ~fxe_batch() {
        if (staged) cudaEventDestroy(staged);
        if (d_hist) cudaFree(d_hist);
        if (d_next) cudaFree(d_next);
        if (d_order) cudaFree(d_order);
        if (d_jobs) cudaFree(d_jobs);
        if (h_jobs) cudaFreeHost(h_jobs);
        if (d_genes) cudaFree(d_genes);
        if (h_genes) cudaFreeHost(h_genes);
        if (d_out) cudaFree(d_out);
        if (h_out) cudaFreeHost(h_out);
        if (stream) cudaStreamDestroy(stream);
    }
};

extern "C" fxe_status fxe_batch_create(int32_t max_jobs, int64_t max_poses, int32_t max_genes, fxe_batch** out) {
    g_err.clear();
    if (!out || max_jobs <= 0 || max_poses <= 0 || max_genes <= 0 || max_poses > (int64_t)1 << 30)
        return fail(FXE_ERR_INVALID_ARGS, "invalid batch limits");
    *out = nullptr;
    int dc = 0;
    if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0) return fail(FXE_ERR_NO_DEVICE, "no CUDA device");
    auto* b = new fxe_batch();
    fxe_status st = [&]() -> fxe_status {
        FXE_TRY(cudaGetDevice(&b->device), "cudaGetDevice");
        b->max_jobs = max_jobs;
        b->max_poses = max_poses;
        b->max_genes = max_genes;
        FXE_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        FXE_TRY(cudaEventCreateWithFlags(&b->staged, cudaEventDisableTiming), "cudaEventCreate");
        FXE_TRY(cudaMalloc(&b->d_jobs, sizeof(fxe::Job) * max_jobs), "batch job table");
        FXE_TRY(cudaMalloc(&b->d_next, sizeof(int)), "batch pose queue");
        FXE_TRY(cudaMalloc(&b->d_order, sizeof(int) * max_poses), "batch pose queue");
        FXE_TRY(fxe::f32::configure_voronoi(), "cudaFuncSetAttribute");
        FXE_TRY(fxe::f64::configure_voronoi(), "cudaFuncSetAttribute");
        b->hist_bytes = fxe::pose_hist_bytes();
        FXE_TRY(cudaMalloc(&b->d_hist, b->hist_bytes + 16), "face history");
        FXE_TRY(cudaMallocHost(&b->h_jobs, sizeof(fxe::Job) * max_jobs), "batch job table");
        FXE_TRY(cudaMalloc(&b->d_genes, sizeof(int32_t) * max_poses * max_genes), "batch staging");
        FXE_TRY(cudaMallocHost(&b->h_genes, sizeof(int32_t) * max_poses * max_genes), "batch staging");
        FXE_TRY(cudaMalloc(&b->d_out, sizeof(fxe_cf) * max_poses), "batch staging");
        FXE_TRY(cudaMallocHost(&b->h_out, sizeof(fxe_cf) * max_poses), "batch staging");
        FXE_TRY(cudaEventRecord(b->staged, b->stream), "cudaEventRecord");
        return FXE_OK;
    }();
    if (st != FXE_OK) {
        delete b;
        return st;
    }
    *out = b;
    return FXE_OK;
}

extern "C" void fxe_batch_destroy(fxe_batch* b) { delete b; }

namespace {

// Fills the job table, uploads it and launches the three kernels over every job's poses.
// genes_of / out_of give each job's device chromosomes and records.
template <typename G, typename O>
fxe_status batch_launch(fxe_batch* b, const fxe_job* jobs, int32_t n_jobs, cudaStream_t s, G genes_of, O out_of) {
    int prec = -1, order = FXE_FACE_ORDER_REFERENCE, total = 0, mobile = 0, cells = -1;
    long long items = 0;
    FXE_TRY(cudaEventSynchronize(b->staged), "batch staging");
    int k = 0;
    for (int i = 0; i < n_jobs; ++i) {
        fxe_context* ctx = jobs[i].ctx;
        if (jobs[i].n == 0) continue;
        fxe::Job& J = b->h_jobs[k++];
        J.S = ctx->S;
        J.W = ctx->W;
        J.W.out = out_of(i);
        J.genes = genes_of(i);
        J.pose0 = total;
        J.n = jobs[i].n;
        J.warp0 = items;
        total += jobs[i].n;
        items += (long long)jobs[i].n * (ctx->S.n_sc + ctx->S.n_lig);
        ctx->last_n = jobs[i].n;
        prec = ctx->precision;
        order = ctx->face_order;
        mobile = std::max(mobile, ctx->S.n_sc + ctx->S.n_lig);
        // the contexts' common cell-staging setting, else the autotuner's choice
        cells = cells < 0 || cells == ctx->cell_staging ? ctx->cell_staging : FXE_CELLS_AUTO;
    }
    if (k == 0) return FXE_OK;
    FXE_TRY(cudaMemcpyAsync(b->d_jobs, b->h_jobs, sizeof(fxe::Job) * k, cudaMemcpyHostToDevice, s), "job table");
    FXE_TRY(cudaEventRecord(b->staged, s), "cudaEventRecord");
    fxe::launch_build_jobs(b->d_jobs, k, total, s);
    fxe::launch_contacts_jobs(b->d_jobs, k, items, s, resolve_staged(cells, prec, mobile, total));
    uint8_t* hist = order == FXE_FACE_ORDER_REFERENCE ? b->d_hist : nullptr;
    const int bpsm = tuned_blocks(prec, mobile, total);
    const fxe::Deal dl = fxe::order_deal(prec, total, hist ? b->hist_bytes : 0, bpsm);
    fxe::launch_order_poses_jobs(b->d_jobs, k, total, b->d_order, s, dl.deal, dl.tile);
    if (prec == FXE_PRECISION_FAST)
        fxe::f32::launch_poses_jobs(b->d_jobs, k, total, b->d_next, b->d_order, hist, b->hist_bytes, bpsm, s);
    else fxe::f64::launch_poses_jobs(b->d_jobs, k, total, b->d_next, b->d_order, hist, b->hist_bytes, bpsm, s);
    FXE_TRY(cudaGetLastError(), "batched kernel launch");
    b->launches += 4;
    return FXE_OK;
}

fxe_status batch_check(fxe_batch* b, const fxe_job* jobs, int32_t n_jobs, bool device_ptrs, int64_t* total) {
    if (!b || (n_jobs > 0 && !jobs) || n_jobs < 0) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    if (n_jobs > b->max_jobs)
        return fail(FXE_ERR_INVALID_ARGS, "n_jobs = " + std::to_string(n_jobs) + " exceeds the batch's max_jobs");
    int64_t t = 0;
    int prec = -1;
    for (int i = 0; i < n_jobs; ++i) {
        const fxe_context* ctx = jobs[i].ctx;
        if (!ctx || jobs[i].n < 0) return fail(FXE_ERR_INVALID_ARGS, "job " + std::to_string(i) + ": no context or n < 0");
        if (jobs[i].n == 0) continue;
        if (!jobs[i].genes || !jobs[i].out) return fail(FXE_ERR_INVALID_ARGS, "job " + std::to_string(i) + ": NULL genes or out");
        if (ctx->device != b->device) return fail(FXE_ERR_INVALID_ARGS, "job " + std::to_string(i) + ": context on another device");
        if (jobs[i].n > ctx->W.max_poses)
            return fail(FXE_ERR_INVALID_ARGS, "job " + std::to_string(i) + ": n exceeds its context's max_poses");
        if (!device_ptrs && ctx->S.n_genes > b->max_genes)
            return fail(FXE_ERR_INVALID_ARGS, "job " + std::to_string(i) + ": more genes than the batch's max_genes");
        if (prec >= 0 && ctx->precision != prec)
            return fail(FXE_ERR_INVALID_ARGS, "jobs of one batch must share one precision");
        prec = ctx->precision;
        for (int q = 0; q < i; ++q)
            if (jobs[q].ctx == ctx && jobs[q].n > 0)
                return fail(FXE_ERR_INVALID_ARGS, "a context appears twice in one batch (its workspace is per context)");
        t += jobs[i].n;
    }
    if (t > b->max_poses) return fail(FXE_ERR_INVALID_ARGS, "total poses exceed the batch's max_poses");
    *total = t;
    return FXE_OK;
}

}  // namespace

extern "C" fxe_status fxe_batch_eval_genes_device(fxe_batch* b, const fxe_job* jobs, int32_t n_jobs, void* stream) {
    g_err.clear();
    int64_t total = 0;
    fxe_status st = batch_check(b, jobs, n_jobs, true, &total);
    if (st != FXE_OK) return st;
    if (cudaSetDevice(b->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    return batch_launch(b, jobs, n_jobs, s, [&](int i) { return (const int32_t*)jobs[i].genes; },
                        [&](int i) { return jobs[i].out; });
}

extern "C" fxe_status fxe_batch_eval_genes(fxe_batch* b, const fxe_job* jobs, int32_t n_jobs) {
    g_err.clear();
    int64_t total = 0;
    fxe_status st = batch_check(b, jobs, n_jobs, false, &total);
    if (st != FXE_OK) return st;
    if (cudaSetDevice(b->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    cudaStream_t s = b->stream;
    // the previous call's copies from the pinned staging have completed (it synchronised)
    std::vector<int64_t> goff(n_jobs + 1, 0), poff(n_jobs + 1, 0);
    for (int i = 0; i < n_jobs; ++i) {
        const int64_t ng = jobs[i].n > 0 ? jobs[i].ctx->S.n_genes : 0;
        goff[i + 1] = goff[i] + (int64_t)jobs[i].n * ng;
        poff[i + 1] = poff[i] + jobs[i].n;
        if (jobs[i].n > 0) std::memcpy(b->h_genes + goff[i], jobs[i].genes, sizeof(int32_t) * jobs[i].n * ng);
    }
    if (total == 0) return FXE_OK;
    FXE_TRY(cudaMemcpyAsync(b->d_genes, b->h_genes, sizeof(int32_t) * goff[n_jobs], cudaMemcpyHostToDevice, s),
            "genes to device");
    st = batch_launch(b, jobs, n_jobs, s, [&](int i) { return (const int32_t*)(b->d_genes + goff[i]); },
                      [&](int i) { return b->d_out + poff[i]; });
    if (st != FXE_OK) return st;
    FXE_TRY(cudaMemcpyAsync(b->h_out, b->d_out, sizeof(fxe_cf) * total, cudaMemcpyDeviceToHost, s), "results to host");
    FXE_TRY(cudaStreamSynchronize(s), "batched evaluation");
    for (int i = 0; i < n_jobs; ++i)
        if (jobs[i].n > 0) std::memcpy(jobs[i].out, b->h_out + poff[i], sizeof(fxe_cf) * jobs[i].n);
    return FXE_OK;
}

extern "C" fxe_status fxe_batch_take_launches(fxe_batch* b, int64_t* launches) {
    g_err.clear();
    if (!b || !launches) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    *launches = b->launches;
    b->launches = 0;
    return FXE_OK;
}

// ------------------------------------------------------------------------------------------
// GA engine: populations resident in HBM; a generation of every running job is one graph of
// breeding, one batched evaluation and selection.
// ------------------------------------------------------------------------------------------
namespace fxe {
void launch_ga_init(const GaJob*, const int*, int, cudaStream_t);
void launch_ga_breed(const GaJob*, const int*, int, cudaStream_t);
void launch_ga_fitness(const GaJob*, const int*, int, bool, cudaStream_t);
void launch_ga_select(GaJob*, const int*, int, bool, cudaStream_t);
}  // namespace fxe

namespace {
struct GaSlot {
    bool used = false, running = false, finished = false;
    fxe_context* ctx = nullptr;
    fxe_ga_job job{};
    int steps = 0;
    std::vector<void*> mem;
    fxe::GaJob J{};   // host copy of the pointers as set up (the device copy swaps them)
};
}  // namespace

struct fxe_ga {
    int device = 0;
    int max_jobs = 0;
    int precision = FXE_PRECISION_REFERENCE;
    cudaStream_t stream = nullptr;
    std::vector<GaSlot> slots;
    fxe::GaJob* d_all = nullptr;        // [max_jobs] per-slot state (pointers swap on device)
    int* d_ids = nullptr;               // [max_jobs] 0..max_jobs-1
    int* d_run = nullptr;               // [max_jobs] running slots of the captured graph
    fxe::Job* d_eval = nullptr;         // [max_jobs] batched-evaluation table of the running slots
    int* d_next = nullptr;              // pose queue of the polyhedron launch
    int* d_order = nullptr;             // its order (order_poses_jobs_kernel)
    int order_cap = 0;
    uint8_t* d_hist = nullptr;          // face history of the polyhedron launch
    size_t hist_bytes = 0;
    std::vector<int> run;               // running slots of the captured graph
    cudaGraphExec_t exec = nullptr;
    bool dirty = true;
    int64_t launches = 0, graph_launches = 0;
    ~fxe_ga() {
        if (stream) cudaStreamSynchronize(stream);
        if (exec) cudaGraphExecDestroy(exec);
        for (auto& s : slots)
            for (void* p : s.mem) cudaFree(p);
        if (d_all) cudaFree(d_all);
        if (d_ids) cudaFree(d_ids);
        if (d_run) cudaFree(d_run);
        if (d_eval) cudaFree(d_eval);
        if (d_next) cudaFree(d_next);
        if (d_order) cudaFree(d_order);
        if (d_hist) cudaFree(d_hist);
        if (stream) cudaStreamDestroy(stream);
    }
};

extern "C" fxe_status fxe_ga_create(int32_t max_jobs, int32_t precision, fxe_ga** out) {
    g_err.clear();
    if (!out || max_jobs <= 0 || (precision != FXE_PRECISION_REFERENCE && precision != FXE_PRECISION_FAST))
        return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    *out = nullptr;
    int dc = 0;
    if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0) return fail(FXE_ERR_NO_DEVICE, "no CUDA device");
    auto* e = new fxe_ga();
    fxe_status st = [&]() -> fxe_status {
        FXE_TRY(cudaGetDevice(&e->device), "cudaGetDevice");
        e->max_jobs = max_jobs;
        e->precision = precision;
        e->slots.resize(max_jobs);
        FXE_TRY(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        FXE_TRY(cudaMalloc(&e->d_all, sizeof(fxe::GaJob) * max_jobs), "GA state");
        FXE_TRY(cudaMalloc(&e->d_ids, sizeof(int) * max_jobs), "GA state");
        FXE_TRY(cudaMalloc(&e->d_run, sizeof(int) * max_jobs), "GA state");
        FXE_TRY(cudaMalloc(&e->d_eval, sizeof(fxe::Job) * max_jobs), "GA state");
        FXE_TRY(cudaMalloc(&e->d_next, sizeof(int)), "GA state");
        FXE_TRY(fxe::f32::configure_voronoi(), "cudaFuncSetAttribute");
        FXE_TRY(fxe::f64::configure_voronoi(), "cudaFuncSetAttribute");
        e->hist_bytes = fxe::pose_hist_bytes();
        FXE_TRY(cudaMalloc(&e->d_hist, e->hist_bytes + 16), "face history");
        std::vector<int> ids(max_jobs);
        for (int i = 0; i < max_jobs; ++i) ids[i] = i;
        FXE_TRY(cudaMemcpy(e->d_ids, ids.data(), sizeof(int) * max_jobs, cudaMemcpyHostToDevice), "GA state");
        return FXE_OK;
    }();
    if (st != FXE_OK) {
        delete e;
        return st;
    }
    *out = e;
    return FXE_OK;
}

extern "C" void fxe_ga_destroy(fxe_ga* e) { delete e; }

namespace {
// Slots of a job's signature set: a power of two at least twice the chromosomes it can take in.
unsigned long long seen_slots(const fxe_ga_job& job) {
    const long long P = job.population, nnew = job.n_new > 0 ? job.n_new : job.population;
    const long long most = P + (long long)(job.generations > 0 ? job.generations : 0) * nnew;
    unsigned long long n = 64;
    while (n < 2ull * (unsigned long long)most) n <<= 1;
    return n;
}
}  // namespace

extern "C" fxe_status fxe_ga_job_bytes(const fxe_ga_job* job, int64_t* bytes) {
    g_err.clear();
    if (!job || !job->ctx || !bytes) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    const int64_t P = job->population, ng = job->ctx->S.n_genes, G = job->generations;
    *bytes = P * ng * 4 * 3 + P * 8 * 2 + P * (int64_t)sizeof(fxe_cf) + G * P * (ng * 4 + 8) + 16 +
             2 * (P + 8) * (ng * 4 + 8) + (job->duplicates ? 0 : 8 * (int64_t)seen_slots(*job)) +
             P * ng * 8 + P * (8 * 3 + 4) + 32 + ng * 4;
    return FXE_OK;
}

extern "C" fxe_status fxe_ga_admit(fxe_ga* e, const fxe_ga_job* job, int32_t* slot_out) {
    g_err.clear();
    if (!e || !job || !job->ctx || !slot_out) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    fxe_context* ctx = job->ctx;
    const int P = job->population, ng = ctx->S.n_genes;
    if (P < 2 || P > 2048 || P > ctx->W.max_poses)
        return fail(FXE_ERR_INVALID_ARGS, "population must be 2..2048 and at most the context's max_poses");
    if (job->generations < 0 || ng < 1 || ng > 64)
        return fail(FXE_ERR_INVALID_ARGS, "generations < 0, or genes outside 1..64");
    const int nnew = job->n_new > 0 ? job->n_new : P;
    if (nnew > P || (job->steady && job->n_new <= 0))
        return fail(FXE_ERR_INVALID_ARGS, "n_new must be 1..population (STEADY needs it set)");
    if (job->fitness != FXE_FITNESS_PSHARE && job->fitness != FXE_FITNESS_LINEAR && job->fitness != FXE_FITNESS_SMFREE)
        return fail(FXE_ERR_INVALID_ARGS, "fitness must be PSHARE, LINEAR or SMFREE");
    if (job->sharing_alpha < 0.0 || job->sharing_peaks < 0.0 || job->sharing_scale < 0.0 ||
        !(job->entropy_weight >= 0.0 && job->entropy_weight <= 1.0))
        return fail(FXE_ERR_INVALID_ARGS, "sharing parameters negative or entropy weight outside [0, 1]");
    if (ctx->device != e->device) return fail(FXE_ERR_INVALID_ARGS, "context on another device");
    for (const auto& s : e->slots)
        if (s.used && s.ctx == ctx) return fail(FXE_ERR_INVALID_ARGS, "the context already runs a job");
    int k = -1;
    for (int i = 0; i < e->max_jobs && k < 0; ++i)
        if (!e->slots[i].used) k = i;
    if (k < 0) return fail(FXE_ERR_OVER_BUDGET, "no free job slot");
    if (cudaSetDevice(e->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    GaSlot& s = e->slots[k];
    auto get = [&](size_t bytes, void** p) -> cudaError_t {
        cudaError_t r = cudaMalloc(p, bytes + 16);
        if (r == cudaSuccess) s.mem.push_back(*p);
        return r;
    };
    fxe::GaJob J{};
    void* q = nullptr;
    fxe_status st = [&]() -> fxe_status {
        FXE_TRY(get(sizeof(int32_t) * P * ng, &q), "GA population"); J.pop = (int32_t*)q;
        FXE_TRY(get(sizeof(int32_t) * P * ng, &q), "GA population"); J.pop_next = (int32_t*)q;
        FXE_TRY(get(sizeof(double) * P, &q), "GA population"); J.pop_e = (double*)q;
        FXE_TRY(get(sizeof(double) * P, &q), "GA population"); J.pop_e_next = (double*)q;
        FXE_TRY(get(sizeof(int32_t) * P * ng, &q), "GA children"); J.child = (int32_t*)q;
        FXE_TRY(get(sizeof(fxe_cf) * P, &q), "GA children"); J.child_cf = (const fxe_cf*)q;
        const size_t G = (size_t)job->generations > 0 ? (size_t)job->generations : 1;
        FXE_TRY(get(sizeof(int32_t) * P * ng * G, &q), "GA snapshots"); J.snap = (int32_t*)q;
        FXE_TRY(get(sizeof(double) * P * G, &q), "GA snapshots"); J.snap_e = (double*)q;
        // gen[0]: generation, gen[1]: pairs in the first candidate batch, gen[2..3]: duplicate
        // counts, gen[4]: signature 0 seen
        FXE_TRY(get(sizeof(int) * 8, &q), "GA counter"); J.gen = (int*)q;
        J.ncand = P + 8;
        const int gen0[8] = {0, std::min(J.ncand, P / 2 + P / 16 + 8), 0, 0, 0, 0, 0, 0};
        FXE_TRY(cudaMemcpyAsync(J.gen, gen0, sizeof(gen0), cudaMemcpyHostToDevice, e->stream), "GA counter");
        FXE_TRY(get(sizeof(int32_t) * 2 * J.ncand * ng, &q), "GA candidates"); J.cand = (int32_t*)q;
        FXE_TRY(get(sizeof(uint64_t) * 2 * J.ncand, &q), "GA candidates"); J.cand_sig = (uint64_t*)q;
        J.reject = job->duplicates ? 0 : 1;
        if (J.reject) {
            const unsigned long long slots = seen_slots(*job);
            FXE_TRY(get(sizeof(uint64_t) * slots, &q), "GA signature set"); J.seen = (uint64_t*)q;
            FXE_TRY(cudaMemsetAsync(J.seen, 0, sizeof(uint64_t) * slots, e->stream), "GA signature set");
            J.hmask = slots - 1;
        }
        J.dec_off = ctx->S.dec_off;
        J.dec_tab = ctx->S.dec_tab;
        J.gene_min = ctx->S.gene_min;
        J.gene_del = ctx->S.gene_del;
        J.gene_max = ctx->S.gene_max;
        {
            // rotamer genes and their side chains' probabilities; like the reference's mutation
            // (genes before num_genes - nflxsc_real, then each rotamer gene) they come last
            std::vector<float> gp(ng, -1.0f);
            std::vector<int> gt(ng), ga(ng);
            FXE_TRY(cudaMemcpy(gt.data(), ctx->S.gene_type, sizeof(int) * ng, cudaMemcpyDeviceToHost), "GA genes");
            FXE_TRY(cudaMemcpy(ga.data(), ctx->S.gene_atom, sizeof(int) * ng, cudaMemcpyDeviceToHost), "GA genes");
            bool seen_rot = false;
            for (int g = 0; g < ng; ++g) {
                if (gt[g] == 4) {
                    gp[g] = ctx->receptor->flex_prob[ga[g]];
                    seen_rot = true;
                } else if (seen_rot) {
                    return fail(FXE_ERR_INVALID_ARGS, "rotamer genes must come after the other genes");
                }
            }
            FXE_TRY(get(sizeof(float) * ng, &q), "GA genes");
            J.gene_prob = (const float*)q;
            FXE_TRY(cudaMemcpyAsync(q, gp.data(), sizeof(float) * ng, cudaMemcpyHostToDevice, e->stream), "GA genes");
            FXE_TRY(cudaStreamSynchronize(e->stream), "GA genes");
        }
        // fitness model; sig_share as LIB/gaboom.cpp:300-309 forms it from the gene limits
        J.fitness = job->fitness;
        const double alpha = job->sharing_alpha > 0.0 ? job->sharing_alpha : 1.0;
        const double peaks = job->sharing_peaks > 0.0 ? job->sharing_peaks : 5.0;
        const double scale = job->sharing_scale > 0.0 ? job->sharing_scale : 10.0;
        double sig = 0.0;
        for (int g = 0; g < ng; ++g) {
            const double w = ctx->h_gmax[g] - ctx->h_gmin[g];
            sig += w * w;
        }
        sig = std::sqrt(sig / (double)ng) / (2.0 * std::pow(peaks, 1.0 / (double)ng));
        J.sig_share = sig / scale;
        J.share_alpha = alpha;
        J.ent_w = job->entropy_weight;
        J.beta = job->temperature > 0.0 ? 1.0 / (0.001987206 * job->temperature) : 0.0;   // kB, LIB/statmech.h:26
        FXE_TRY(get(sizeof(double) * P * ng, &q), "GA fitness"); J.pic = (double*)q;
        FXE_TRY(get(sizeof(double) * P, &q), "GA fitness"); J.share = (double*)q;
        FXE_TRY(get(sizeof(double) * P, &q), "GA fitness"); J.fit = (double*)q;
        FXE_TRY(get(sizeof(double) * P, &q), "GA fitness"); J.fcum = (double*)q;
        FXE_TRY(get(sizeof(int) * P, &q), "GA fitness"); J.ford = (int*)q;
        FXE_TRY(get(sizeof(double) * 4, &q), "GA fitness"); J.fstat = (double*)q;
        J.seed = job->seed;
        J.cross_rate = job->cross_rate;
        J.mut_rate = job->mut_rate;
        J.P = P;
        J.ng = ng;
        J.G = job->generations;
        J.nnew = nnew;
        J.steady = job->steady ? 1 : 0;
        J.intragenes = job->intragenes ? 1 : 0;
        J.adaptive = job->adaptive ? 1 : 0;
        for (int q = 0; q < 4; ++q) J.k[q] = job->k[q];
        FXE_TRY(cudaMemcpyAsync(e->d_all + k, &J, sizeof(J), cudaMemcpyHostToDevice, e->stream), "GA state");
        // generation 0: uniform genes, evaluated on the job's context, sorted
        fxe::launch_ga_init(e->d_all, e->d_ids + k, 1, e->stream);
        const int prec = ctx->precision;
        ctx->precision = e->precision;
        fxe_status r = run_chunk(ctx, P, J.child, nullptr, e->stream);
        ctx->precision = prec;
        if (r != FXE_OK) return r;
        FXE_TRY(cudaMemcpyAsync((void*)J.child_cf, ctx->W.out, sizeof(fxe_cf) * P, cudaMemcpyDeviceToDevice, e->stream),
                "GA records");
        fxe::launch_ga_select(e->d_all, e->d_ids + k, 1, true, e->stream);
        fxe::launch_ga_fitness(e->d_all, e->d_ids + k, 1, true, e->stream);
        FXE_TRY(cudaGetLastError(), "GA launch");
        FXE_TRY(cudaStreamSynchronize(e->stream), "GA admission");   // gen0 and the host copy of J die here
        e->launches += 10;
        return FXE_OK;
    }();
    if (st != FXE_OK) {
        for (void* p : s.mem) cudaFree(p);
        s.mem.clear();
        return st;
    }
    s.used = true;
    s.running = job->generations > 0;
    s.finished = job->generations == 0;
    s.ctx = ctx;
    s.job = *job;
    s.steps = 0;
    s.J = J;
    e->dirty = true;
    *slot_out = k;
    return FXE_OK;
}

extern "C" fxe_status fxe_ga_step(fxe_ga* e) {
    g_err.clear();
    if (!e) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    if (cudaSetDevice(e->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    if (e->dirty) {
        e->run.clear();
        for (int i = 0; i < e->max_jobs; ++i)
            if (e->slots[i].running) e->run.push_back(i);
        if (e->exec) {
            cudaGraphExecDestroy(e->exec);
            e->exec = nullptr;
        }
        e->dirty = false;
        if (e->run.empty()) return FXE_OK;
        const int n = (int)e->run.size();
        std::vector<fxe::Job> ev(n);
        int total = 0;
        long long items = 0;
        for (int r = 0; r < n; ++r) {
            GaSlot& s = e->slots[e->run[r]];
            fxe::Job& J = ev[r];
            J.S = s.ctx->S;
            J.W = s.ctx->W;
            J.W.out = const_cast<fxe_cf*>(s.J.child_cf);
            J.genes = s.J.child;
            J.pose0 = total;
            J.n = s.J.nnew;
            J.warp0 = items;
            total += J.n;
            items += (long long)J.n * (s.ctx->S.n_sc + s.ctx->S.n_lig);
        }
        if (total > e->order_cap) {   // the pose order of the polyhedron launch, sized for the running jobs
            FXE_TRY(cudaStreamSynchronize(e->stream), "GA table");
            if (e->d_order) cudaFree(e->d_order);
            e->d_order = nullptr;
            e->order_cap = 0;
            FXE_TRY(cudaMalloc(&e->d_order, sizeof(int) * total), "GA pose order");
            e->order_cap = total;
        }
        FXE_TRY(cudaMemcpyAsync(e->d_run, e->run.data(), sizeof(int) * n, cudaMemcpyHostToDevice, e->stream), "GA table");
        FXE_TRY(cudaMemcpyAsync(e->d_eval, ev.data(), sizeof(fxe::Job) * n, cudaMemcpyHostToDevice, e->stream), "GA table");
        FXE_TRY(cudaStreamSynchronize(e->stream), "GA table");
        cudaGraph_t g = nullptr;
        FXE_TRY(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
        fxe::launch_ga_breed(e->d_all, e->d_run, n, e->stream);
        fxe::launch_build_jobs(e->d_eval, n, total, e->stream);
        // the running jobs' largest scored-atom count, and their common cell-staging setting
        int mobile = 0, cells = -1;
        for (int sl : e->run) {
            const fxe_context* c = e->slots[sl].ctx;
            mobile = std::max(mobile, c->S.n_sc + c->S.n_lig);
            cells = cells < 0 || cells == c->cell_staging ? c->cell_staging : FXE_CELLS_AUTO;
        }
        fxe::launch_contacts_jobs(e->d_eval, n, items, e->stream, resolve_staged(cells, e->precision, mobile, total));
        // the GA engine keeps the reference's face order unless a running job's context asks otherwise
        bool ref_order = true;
        for (int sl : e->run) ref_order = ref_order && e->slots[sl].ctx->face_order == FXE_FACE_ORDER_REFERENCE;
        uint8_t* hist = ref_order ? e->d_hist : nullptr;
        const int bpsm = tuned_blocks(e->precision, mobile, total);
        const fxe::Deal dl = fxe::order_deal(e->precision, total, hist ? e->hist_bytes : 0, bpsm);
        fxe::launch_order_poses_jobs(e->d_eval, n, total, e->d_order, e->stream, dl.deal, dl.tile);
        if (e->precision == FXE_PRECISION_FAST)
            fxe::f32::launch_poses_jobs(e->d_eval, n, total, e->d_next, e->d_order, hist, e->hist_bytes, bpsm, e->stream);
        else fxe::f64::launch_poses_jobs(e->d_eval, n, total, e->d_next, e->d_order, hist, e->hist_bytes, bpsm,
                                         e->stream);
        fxe::launch_ga_select(e->d_all, e->d_run, n, false, e->stream);
        fxe::launch_ga_fitness(e->d_all, e->d_run, n, false, e->stream);
        cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
        if (ce != cudaSuccess) return cuda_fail(ce, "graph capture");
        ce = cudaGraphInstantiate(&e->exec, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return cuda_fail(ce, "graph instantiate");
    }
    if (e->run.empty()) return FXE_OK;
    FXE_TRY(cudaGraphLaunch(e->exec, e->stream), "graph launch");
    e->launches += 10;
    e->graph_launches += 1;
    for (int i : e->run) {
        GaSlot& s = e->slots[i];
        if (++s.steps >= s.job.generations) {
            s.running = false;
            s.finished = true;
            e->dirty = true;
        }
    }
    return FXE_OK;
}

extern "C" fxe_status fxe_ga_finished(fxe_ga* e, int32_t* slots, int32_t cap, int32_t* n) {
    g_err.clear();
    if (!e || !n || cap < 0 || (cap > 0 && !slots)) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    FXE_TRY(cudaStreamSynchronize(e->stream), "GA step");
    int k = 0;
    for (int i = 0; i < e->max_jobs; ++i)
        if (e->slots[i].used && e->slots[i].finished) {
            if (k < cap) slots[k] = i;
            ++k;
        }
    *n = k;
    return FXE_OK;
}

namespace {
// The ensemble of a job as the reference's GA assembles it (LIB/gaboom.cpp:520-540), on the
// device (fxe_ensemble.cu): every generation's population, sorted by energy (ties in snapshot
// order), chromosomes within 0.1 of the last one kept on every decoded gene dropped (remove_dups,
// :2728-2747). Leaves the kept energies (energy order) in *d_e and, when want_ic, their decoded
// ICs (clamped as eval_chromosome leaves them) in *d_ic; both are freed with `bufs`.
fxe_status ga_ensemble(const GaSlot& s, const fxe::GaJob& J, cudaStream_t st, bool want_ic, CallBuffers& bufs,
                       double** d_e, double** d_ic, int64_t* n_kept) {
    const int P = s.job.population, ng = s.ctx->S.n_genes, G = s.job.generations;
    const long long N = (long long)G * P;
    if (N >= (1ll << 31)) return fail(FXE_ERR_CAPACITY, "ensemble larger than 2^31 chromosomes");
    *n_kept = 0;
    *d_e = nullptr;
    if (d_ic) *d_ic = nullptr;
    if (N == 0) return FXE_OK;
    void* scratch = nullptr;
    int* d_cnt = nullptr;
    FXE_TRY(bufs.get(reinterpret_cast<unsigned char**>(&scratch), fxe::ensemble_scratch_bytes(N, ng)), "ensemble scratch");
    FXE_TRY(bufs.get(d_e, (size_t)N), "ensemble output");
    if (want_ic) FXE_TRY(bufs.get(d_ic, (size_t)N * ng), "ensemble output");
    FXE_TRY(bufs.get(&d_cnt, 1), "ensemble output");
    FXE_TRY(fxe::launch_ensemble(N, ng, J.snap_e, nullptr, &s.ctx->S, J.snap, scratch, nullptr, *d_e,
                                 want_ic ? *d_ic : nullptr, d_cnt, st), "ensemble launch");
    int cnt = 0;
    FXE_TRY(cudaMemcpyAsync(&cnt, d_cnt, sizeof(int), cudaMemcpyDeviceToHost, st), "ensemble size");
    FXE_TRY(cudaStreamSynchronize(st), "ensemble");
    if (cnt < 0 || cnt > N) return fail(FXE_ERR_INTERNAL, "ensemble size out of range");
    *n_kept = cnt;
    return FXE_OK;
}

}  // namespace

extern "C" fxe_status fxe_ga_collect(fxe_ga* e, int32_t slot, double temperature, int32_t* best_genes,
                                     double* best_energy, fxe_thermo* thermo, int64_t* n_ensemble) {
    g_err.clear();
    if (!e || slot < 0 || slot >= e->max_jobs || !e->slots[slot].used || !e->slots[slot].finished)
        return fail(FXE_ERR_INVALID_ARGS, "slot does not hold a finished job");
    GaSlot& s = e->slots[slot];
    if (cudaSetDevice(e->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    FXE_TRY(cudaStreamSynchronize(e->stream), "GA step");
    fxe::GaJob J;
    FXE_TRY(cudaMemcpy(&J, e->d_all + slot, sizeof(J), cudaMemcpyDeviceToHost), "GA state");
    const int ng = s.ctx->S.n_genes;
    if (best_genes) FXE_TRY(cudaMemcpy(best_genes, J.pop, sizeof(int32_t) * ng, cudaMemcpyDeviceToHost), "GA result");
    if (best_energy) FXE_TRY(cudaMemcpy(best_energy, J.pop_e, sizeof(double), cudaMemcpyDeviceToHost), "GA result");
    if (thermo || n_ensemble) {
        CallBuffers bufs;
        double* d_e = nullptr;
        int64_t nk = 0;
        fxe_status st = ga_ensemble(s, J, e->stream, false, bufs, &d_e, nullptr, &nk);
        if (st != FXE_OK) return st;
        if (n_ensemble) *n_ensemble = nk;
        if (thermo) {
            if (nk == 0) return fail(FXE_ERR_INVALID_ARGS, "the job ran no generation: empty ensemble");
            if (!(temperature > 0.0)) return fail(FXE_ERR_INVALID_ARGS, "temperature must be positive");
            st = thermo_run(d_e, nullptr, (long)nk, temperature, thermo, nullptr, e->stream);
            if (st != FXE_OK) return st;
        }
    }
    for (void* p : s.mem) cudaFree(p);
    s = GaSlot();
    return FXE_OK;
}

extern "C" fxe_status fxe_ga_ensemble(fxe_ga* e, int32_t slot, int64_t cap, double* ic, double* energies,
                                      int64_t* n) {
    g_err.clear();
    if (!e || !n || slot < 0 || slot >= e->max_jobs || !e->slots[slot].used || !e->slots[slot].finished)
        return fail(FXE_ERR_INVALID_ARGS, "slot does not hold a finished job");
    GaSlot& s = e->slots[slot];
    if (cudaSetDevice(e->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    FXE_TRY(cudaStreamSynchronize(e->stream), "GA step");
    fxe::GaJob J;
    FXE_TRY(cudaMemcpy(&J, e->d_all + slot, sizeof(J), cudaMemcpyDeviceToHost), "GA state");
    CallBuffers bufs;
    double *d_e = nullptr, *d_ic = nullptr;
    fxe_status st = ga_ensemble(s, J, e->stream, ic != nullptr, bufs, &d_e, &d_ic, n);
    if (st != FXE_OK) return st;
    if (!ic && !energies) return FXE_OK;
    if (cap < *n) return fail(FXE_ERR_CAPACITY, "the ensemble holds more chromosomes than cap");
    const int ng = s.ctx->S.n_genes;
    if (*n > 0) {
        if (ic) FXE_TRY(cudaMemcpyAsync(ic, d_ic, sizeof(double) * (size_t)*n * ng, cudaMemcpyDeviceToHost, e->stream), "ensemble ICs");
        if (energies) FXE_TRY(cudaMemcpyAsync(energies, d_e, sizeof(double) * (size_t)*n, cudaMemcpyDeviceToHost, e->stream), "ensemble energies");
        FXE_TRY(cudaStreamSynchronize(e->stream), "ensemble");
    }
    return FXE_OK;
}

extern "C" fxe_status fxe_ga_duplicates(fxe_ga* e, int32_t slot, int64_t* rejected, int64_t* forced) {
    g_err.clear();
    if (!e || slot < 0 || slot >= e->max_jobs || !e->slots[slot].used) return fail(FXE_ERR_INVALID_ARGS, "empty slot");
    if (cudaSetDevice(e->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    FXE_TRY(cudaStreamSynchronize(e->stream), "GA step");
    int gen[4];
    FXE_TRY(cudaMemcpy(gen, e->slots[slot].J.gen, sizeof(gen), cudaMemcpyDeviceToHost), "GA counter");
    if (rejected) *rejected = gen[3];
    if (forced) *forced = gen[2];
    return FXE_OK;
}

extern "C" fxe_status fxe_ga_take_launches(fxe_ga* e, int64_t* launches, int64_t* graphs) {
    g_err.clear();
    if (!e) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    if (launches) *launches = e->launches;
    if (graphs) *graphs = e->graph_launches;
    e->launches = e->graph_launches = 0;
    return FXE_OK;
}

extern "C" fxe_status fxe_ga_population(fxe_ga* e, int32_t slot, int32_t* genes, double* energies) {
    g_err.clear();
    if (!e || slot < 0 || slot >= e->max_jobs || !e->slots[slot].used) return fail(FXE_ERR_INVALID_ARGS, "empty slot");
    GaSlot& s = e->slots[slot];
    if (cudaSetDevice(e->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    FXE_TRY(cudaStreamSynchronize(e->stream), "GA step");
    fxe::GaJob J;
    FXE_TRY(cudaMemcpy(&J, e->d_all + slot, sizeof(J), cudaMemcpyDeviceToHost), "GA state");
    const int P = s.job.population, ng = s.ctx->S.n_genes;
    if (genes) FXE_TRY(cudaMemcpy(genes, J.pop, sizeof(int32_t) * P * ng, cudaMemcpyDeviceToHost), "GA population");
    if (energies) FXE_TRY(cudaMemcpy(energies, J.pop_e, sizeof(double) * P, cudaMemcpyDeviceToHost), "GA population");
    return FXE_OK;
}

// ------------------------------------------------------------------------------------------
// The GA operators and the gene decoder on caller-given inputs.
// ------------------------------------------------------------------------------------------
namespace fxe {
void launch_decode(const DevSystem&, long long, const int32_t*, double*, int, cudaStream_t);
void launch_ga_breed_draws(const GaJob*, const double*, long long, int, int*, cudaStream_t);
void launch_ga_niche(const GaJob*, const int*, cudaStream_t);
}  // namespace fxe


extern "C" fxe_status fxe_decode_genes(fxe_context* ctx, int64_t n, const int32_t* genes, int32_t clamp, double* ic) {
    g_err.clear();
    if (!ctx || n < 0 || (n > 0 && (!genes || !ic))) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    if (n == 0 || ctx->S.n_genes == 0) return FXE_OK;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    const size_t cnt = (size_t)n * ctx->S.n_genes;
    CallBuffers b;
    int32_t* d_g = nullptr;
    double* d_ic = nullptr;
    FXE_TRY(b.put(&d_g, genes, cnt), "genes to device");
    FXE_TRY(b.get(&d_ic, cnt), "decode buffer");
    fxe::launch_decode(ctx->S, n, d_g, d_ic, clamp ? 1 : 0, ctx->stream);
    FXE_TRY(cudaGetLastError(), "decode launch");
    FXE_TRY(cudaMemcpyAsync(ic, d_ic, cnt * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "ICs to host");
    FXE_TRY(cudaStreamSynchronize(ctx->stream), "decode");
    return FXE_OK;
}

extern "C" fxe_status fxe_ga_breed_draws(int32_t population, int32_t n_genes, const int32_t* pop,
                                         const double* fitness, const int32_t* order, const float* gene_prob,
                                         double cross_rate, double mut_rate, int32_t intragenes, int32_t adaptive,
                                         const double* k4, int32_t n_pairs, const double* draws, int32_t* children,
                                         int32_t* draws_used, double* fit_stats) {
    g_err.clear();
    const int P = population, ng = n_genes;
    if (P < 1 || ng < 1 || ng > 1024 || n_pairs < 0 || !pop || !fitness || (n_pairs > 0 && (!draws || !children)) ||
        (adaptive && !k4))
        return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    std::vector<int32_t> ord(P);
    for (int i = 0; i < P; ++i) {
        ord[i] = order ? order[i] : i;
        if (ord[i] < 0 || ord[i] >= P) return fail(FXE_ERR_INVALID_ARGS, "order names no chromosome");
    }
    std::vector<float> prob(ng, -1.0f);
    if (gene_prob)
        for (int q = 0; q < ng; ++q) prob[q] = gene_prob[q];
    int dc = 0;
    if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0) return fail(FXE_ERR_NO_DEVICE, "no CUDA device");
    const long long stride = FXE_GA_DRAWS_PER_PAIR(ng);
    CallBuffers b;
    fxe::GaJob J{};
    J.P = P;
    J.ng = ng;
    J.cross_rate = cross_rate;
    J.mut_rate = mut_rate;
    J.intragenes = intragenes ? 1 : 0;
    J.adaptive = adaptive ? 1 : 0;
    for (int i = 0; i < 4; ++i) J.k[i] = adaptive ? k4[i] : 0.0;
    const int np = n_pairs > 0 ? n_pairs : 1;
    int32_t* d_pop = nullptr;
    double* d_fit = nullptr;
    int* d_ord = nullptr;
    float* d_prob = nullptr;
    FXE_TRY(b.put(&d_pop, pop, (size_t)P * ng), "GA buffers");
    FXE_TRY(b.put(&d_fit, fitness, (size_t)P), "GA buffers");
    FXE_TRY(b.put(&d_ord, ord.data(), (size_t)P), "GA buffers");
    FXE_TRY(b.put(&d_prob, prob.data(), (size_t)ng), "GA buffers");
    J.pop = d_pop;
    J.fit = d_fit;
    J.ford = d_ord;
    J.gene_prob = d_prob;
    FXE_TRY(b.get(&J.fcum, (size_t)P), "GA buffers");
    FXE_TRY(b.get(&J.fstat, 4), "GA buffers");
    FXE_TRY(b.get(&J.child, (size_t)2 * np * ng), "GA buffers");
    double* d_draws = nullptr;
    int* d_used = nullptr;
    FXE_TRY(b.get(&d_used, (size_t)np), "GA buffers");
    if (n_pairs > 0) FXE_TRY(b.put(&d_draws, draws, (size_t)n_pairs * stride), "draws to device");
    fxe::GaJob* d_J = nullptr;
    FXE_TRY(b.put(&d_J, &J, 1), "GA state");
    fxe::launch_ga_breed_draws(d_J, d_draws, stride, n_pairs, d_used, nullptr);
    FXE_TRY(cudaGetLastError(), "GA launch");
    FXE_TRY(cudaDeviceSynchronize(), "GA breeding");
    if (n_pairs > 0) {
        FXE_TRY(cudaMemcpy(children, J.child, sizeof(int32_t) * 2 * (size_t)n_pairs * ng, cudaMemcpyDeviceToHost),
                "children to host");
        std::vector<int> used(n_pairs);
        FXE_TRY(cudaMemcpy(used.data(), d_used, sizeof(int) * n_pairs, cudaMemcpyDeviceToHost), "draw counts");
        for (int k = 0; k < n_pairs; ++k) {
            if (used[k] < 0) return fail(FXE_ERR_INVALID_ARGS, "pair " + std::to_string(k) + " needed more draws than a row holds");
            if (draws_used) draws_used[k] = used[k];
        }
    }
    if (fit_stats) {
        double st[4];
        FXE_TRY(cudaMemcpy(st, J.fstat, sizeof(st), cudaMemcpyDeviceToHost), "fitness stats");
        fit_stats[0] = st[0];
        fit_stats[1] = st[1];
        fit_stats[2] = st[2];
    }
    return FXE_OK;
}

extern "C" fxe_status fxe_ga_niche_counts(int32_t population, int32_t n_genes, const double* ic, double sig_share,
                                          double alpha, double* share) {
    g_err.clear();
    const int P = population, ng = n_genes;
    if (P < 1 || P > 2048 || ng < 1 || !ic || !share || !(sig_share > 0.0))
        return fail(FXE_ERR_INVALID_ARGS, "invalid arguments (population 1..2048, sig_share > 0)");
    int dc = 0;
    if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0) return fail(FXE_ERR_NO_DEVICE, "no CUDA device");
    CallBuffers b;
    fxe::GaJob J{};
    J.P = P;
    J.ng = ng;
    J.fitness = fxe::kFitPshare;
    J.sig_share = sig_share;
    J.share_alpha = alpha;
    double* d_ic = nullptr;
    FXE_TRY(b.put(&d_ic, ic, (size_t)P * ng), "ICs to device");
    J.pic = d_ic;
    FXE_TRY(b.get(&J.share, (size_t)P), "niche buffer");
    fxe::GaJob* d_J = nullptr;
    FXE_TRY(b.put(&d_J, &J, 1), "GA state");
    const int zero = 0;
    int* d_run = nullptr;
    FXE_TRY(b.put(&d_run, &zero, 1), "GA state");
    fxe::launch_ga_niche(d_J, d_run, nullptr);
    FXE_TRY(cudaGetLastError(), "niche launch");
    FXE_TRY(cudaDeviceSynchronize(), "niche counts");
    FXE_TRY(cudaMemcpy(share, J.share, sizeof(double) * P, cudaMemcpyDeviceToHost), "niche counts to host");
    return FXE_OK;
}

extern "C" fxe_status fxe_ensemble_dedup(int64_t n, int32_t n_genes, const double* ic, const double* energies,
                                         int64_t* kept_index, double* kept_energy, int64_t* n_kept) {
    g_err.clear();
    if (n < 0 || n >= ((int64_t)1 << 31) || n_genes < 1 || !n_kept || (n > 0 && (!ic || !energies)))
        return fail(FXE_ERR_INVALID_ARGS, "invalid arguments (0 <= n < 2^31, n_genes >= 1)");
    *n_kept = 0;
    if (n == 0) return FXE_OK;
    int dc = 0;
    if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0) return fail(FXE_ERR_NO_DEVICE, "no CUDA device");
    CallBuffers b;
    double *d_ic = nullptr, *d_e = nullptr, *d_eo = nullptr;
    long long* d_idx = nullptr;
    unsigned char* scratch = nullptr;
    int* d_cnt = nullptr;
    FXE_TRY(b.put(&d_ic, ic, (size_t)n * n_genes), "ensemble input");
    FXE_TRY(b.put(&d_e, energies, (size_t)n), "ensemble input");
    FXE_TRY(b.get(&d_eo, (size_t)n), "ensemble output");
    FXE_TRY(b.get(&d_idx, (size_t)n), "ensemble output");
    FXE_TRY(b.get(&d_cnt, 1), "ensemble output");
    FXE_TRY(b.get(&scratch, fxe::ensemble_scratch_bytes(n, n_genes)), "ensemble scratch");
    FXE_TRY(fxe::launch_ensemble(n, n_genes, d_e, d_ic, nullptr, nullptr, scratch, d_idx, d_eo, nullptr, d_cnt, nullptr),
            "ensemble launch");
    int cnt = 0;
    FXE_TRY(cudaMemcpy(&cnt, d_cnt, sizeof(int), cudaMemcpyDeviceToHost), "ensemble size");
    if (cnt < 0 || cnt > n) return fail(FXE_ERR_INTERNAL, "ensemble size out of range");
    *n_kept = cnt;
    if (cnt > 0 && kept_index) {
        std::vector<long long> idx(cnt);
        FXE_TRY(cudaMemcpy(idx.data(), d_idx, sizeof(long long) * cnt, cudaMemcpyDeviceToHost), "kept indices");
        for (int i = 0; i < cnt; ++i) kept_index[i] = idx[i];
    }
    if (cnt > 0 && kept_energy) FXE_TRY(cudaMemcpy(kept_energy, d_eo, sizeof(double) * cnt, cudaMemcpyDeviceToHost), "kept energies");
    return FXE_OK;
}

extern "C" fxe_status fxe_cleft_grid(int32_t n_spheres, const float* centers, const float* radii, float spacing,
                                     const float* ori, int64_t cap, float* xyz, float* ic, int64_t* n_points) {
    g_err.clear();
    if (n_spheres < 1 || !centers || !radii || !ori || !n_points || !(spacing > 0.0f) || cap < 0 ||
        (cap > 0 && !xyz))
        return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    *n_points = 0;
    // the lattice of each sphere as generate_grid walks it (LIB/generate_grid.cpp:34-95), in float
    const bool fractional = (float)(1.0 / spacing) - (float)((int)(1.0 / spacing)) > 0.001;
    std::vector<float> axes, sph;
    std::vector<long long> off;
    std::vector<int> dims;
    long long max_lattice = 0, total = 0;
    for (int s = 0; s < n_spheres; ++s) {
        const float r = radii[s];
        if (!(r > 0.0f) || r > 1000.0f) return fail(FXE_ERR_INVALID_ARGS, "sphere radius outside (0, 1000] A");
        off.push_back((long long)axes.size());
        int n3[3];
        for (int k = 0; k < 3; ++k) {
            const float c = centers[3 * s + k];
            if (!(c > -1000.0f && c < 1000.0f)) return fail(FXE_ERR_INVALID_ARGS, "sphere centre outside +-1000 A");
            float mn, mx;
            if (fractional) {
                mn = (float)((int)((c - r) / spacing)) * spacing;
                mx = (float)((int)((c + r) / spacing) + 1.0) * spacing;
            } else {
                mn = (float)((int)(c - r - spacing));
                mx = (float)((int)(c + r + spacing) + 1.0);
            }
            int n = 0;
            for (float v = mn; v < mx; v += spacing) {
                axes.push_back(v);
                if (++n > (1 << 20)) return fail(FXE_ERR_INVALID_ARGS, "lattice too large");
            }
            n3[k] = n;
        }
        dims.insert(dims.end(), n3, n3 + 3);
        sph.insert(sph.end(), {centers[3 * s], centers[3 * s + 1], centers[3 * s + 2], r * r});
        const long long lat = (long long)n3[0] * n3[1] * n3[2];
        if (lat >= (1ll << 31)) return fail(FXE_ERR_INVALID_ARGS, "lattice too large");
        max_lattice = lat > max_lattice ? lat : max_lattice;
        total += lat;
    }
    int dc = 0;
    if (cudaGetDeviceCount(&dc) != cudaSuccess || dc == 0) return fail(FXE_ERR_NO_DEVICE, "no CUDA device");
    long long slots = 1024;
    while (slots < 2 * total) slots <<= 1;
    CallBuffers b;
    float *d_axes = nullptr, *d_xyz = nullptr, *d_ic = nullptr;
    unsigned char* scratch = nullptr;
    FXE_TRY(b.put(&d_axes, axes.data(), axes.size()), "grid axes");
    FXE_TRY(b.get(&d_xyz, (size_t)3 * (total > 0 ? total : 1)), "grid points");
    FXE_TRY(b.get(&scratch, fxe::grid_scratch_bytes(max_lattice, slots)), "grid scratch");
    cudaStream_t st = nullptr;
    FXE_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
    long long n = 0;
    cudaError_t e = fxe::launch_cleft_grid(n_spheres, d_axes, off.data(), dims.data(), sph.data(), max_lattice, slots,
                                           scratch, d_xyz, &n, st);
    if (e == cudaSuccess && n > 0 && ic) {
        e = cudaMalloc(reinterpret_cast<void**>(&d_ic), (size_t)3 * n * sizeof(float) + 16);
        if (e == cudaSuccess) {
            b.p.push_back(d_ic);
            fxe::launch_cleft_ic(d_xyz, n, ori, d_ic, st);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess && n > 0 && n <= cap) {
        e = cudaMemcpyAsync(xyz, d_xyz, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && ic) e = cudaMemcpyAsync(ic, d_ic, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return cuda_fail(e, "cleft grid");
    *n_points = n;
    if (n > cap) return fail(FXE_ERR_CAPACITY, "the grid holds more points than cap");
    return FXE_OK;
}

// The autotuner's sweep: times the polyhedron launch over the context's batch at every cap from
// half the SM's capacity to all of it; fills caps/ms (up to max_out entries, may be null) and
// records the fastest cap for the context's size class.
static fxe_status autotune_sweep(fxe_context* ctx, int32_t n, const int32_t* d_genes, int32_t reps, int32_t* caps,
                                 double* ms_out, int32_t max_out, int32_t* n_out, int32_t* blocks_per_sm,
                                 double* ms_per_launch) {
    g_err.clear();
    if (!ctx || n <= 0 || !d_genes || reps < 1 || reps > 100 || max_out < 0)
        return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    if (n > ctx->W.max_poses) return fail(FXE_ERR_INVALID_ARGS, "n exceeds the context's max_poses");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    cudaStream_t s = ctx->stream;
    const bool fast = ctx->precision == FXE_PRECISION_FAST;
    const int maxb = fast ? fxe::f32::pose_max_blocks_per_sm() : fxe::f64::pose_max_blocks_per_sm();
    uint8_t* hist = ctx->face_order == FXE_FACE_ORDER_REFERENCE ? ctx->d_hist : nullptr;
    // the candidates' work: this batch built, its contact candidates listed and ordered once
    fxe::launch_build(ctx->S, ctx->W, n, d_genes, nullptr, s);
    fxe::launch_contacts(ctx->S, ctx->W, n, s, false);
    const fxe::Deal dl = fxe::order_deal(ctx->precision, n, hist ? ctx->hist_bytes : 0, 0);
    fxe::launch_order_poses(ctx->S, ctx->W, n, s, dl.deal, dl.tile);
    FXE_TRY(cudaGetLastError(), "autotune launch");
    cudaEvent_t a = nullptr, b = nullptr;
    FXE_TRY(cudaEventCreate(&a), "cudaEventCreate");
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return fail(FXE_ERR_LAUNCH, "cudaEventCreate");
    }
    int best = 0, n_done = 0;
    float best_ms = 0.0f;
    cudaError_t e = cudaSuccess;
    for (int c = std::max(1, maxb / 2); c <= maxb && e == cudaSuccess; ++c) {
        float cand = 0.0f;
        for (int r = 0; r <= reps && e == cudaSuccess; ++r) {   // the first launch warms up
            cudaEventRecord(a, s);
            if (fast) fxe::f32::launch_poses(ctx->S, ctx->W, n, ctx->W.counters + 4, hist, ctx->hist_bytes, c, s);
            else fxe::f64::launch_poses(ctx->S, ctx->W, n, ctx->W.counters + 4, hist, ctx->hist_bytes, c, s);
            cudaEventRecord(b, s);
            e = cudaEventSynchronize(b);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
            if (r > 0 && (cand == 0.0f || ms < cand)) cand = ms;
        }
        if (e != cudaSuccess) break;
        if (n_done < max_out) {
            if (caps) caps[n_done] = c;
            if (ms_out) ms_out[n_done] = cand;
            ++n_done;
        }
        if (best == 0 || cand < best_ms) {
            best = c;
            best_ms = cand;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (e != cudaSuccess) return cuda_fail(e, "autotune");
    ctx->launches += 3 + (long long)(maxb - std::max(1, maxb / 2) + 1) * (reps + 1);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[size_class(ctx->precision, ctx->S.n_sc + ctx->S.n_lig, n)].blocks = best;
    }
    if (n_out) *n_out = n_done;
    if (blocks_per_sm) *blocks_per_sm = best;
    if (ms_per_launch) *ms_per_launch = best_ms;
    return FXE_OK;
}

// The contact-candidate launch over the context's built batch of n poses timed in both forms
// (rigid cell entries read in place, and staged in shared memory), reps timed launches each after
// one warm-up; records the faster form for the context's size class. ms2: the two fastest times.
static fxe_status tune_contacts(fxe_context* ctx, int32_t n, int32_t reps, double* ms2, int32_t* staged) {
    cudaStream_t s = ctx->stream;
    cudaEvent_t a = nullptr, b = nullptr;
    FXE_TRY(cudaEventCreate(&a), "cudaEventCreate");
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return fail(FXE_ERR_LAUNCH, "cudaEventCreate");
    }
    float best[2] = {0.0f, 0.0f};
    cudaError_t e = cudaSuccess;
    for (int form = 0; form < 2 && e == cudaSuccess; ++form) {
        for (int r = 0; r <= reps && e == cudaSuccess; ++r) {   // the first launch warms up
            cudaEventRecord(a, s);
            fxe::launch_contacts(ctx->S, ctx->W, n, s, form == 1);
            cudaEventRecord(b, s);
            e = cudaEventSynchronize(b);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
            if (r > 0 && (best[form] == 0.0f || ms < best[form])) best[form] = ms;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (e != cudaSuccess) return cuda_fail(e, "autotune");
    ctx->launches += 2LL * (reps + 1);
    const bool st = best[1] < best[0];
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[size_class(ctx->precision, ctx->S.n_sc + ctx->S.n_lig, n)].staged = st ? 1 : 0;
    }
    if (ms2) {
        ms2[0] = best[0];
        ms2[1] = best[1];
    }
    if (staged) *staged = st ? 1 : 0;
    return FXE_OK;
}

extern "C" fxe_status fxe_context_autotune(fxe_context* ctx, int32_t n, const int32_t* d_genes, int32_t reps,
                                           int32_t* blocks_per_sm, double* ms_per_launch) {
    const fxe_status st = autotune_sweep(ctx, n, d_genes, reps, nullptr, nullptr, 0, nullptr, blocks_per_sm,
                                         ms_per_launch);
    if (st != FXE_OK) return st;
    return tune_contacts(ctx, n, reps, nullptr, nullptr);
}

extern "C" fxe_status fxe_context_autotune_contacts(fxe_context* ctx, int32_t n, const int32_t* d_genes, int32_t reps,
                                                    double* ms2, int32_t* staged) {
    g_err.clear();
    if (!ctx || n <= 0 || !d_genes || reps < 1 || reps > 100) return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    if (n > ctx->W.max_poses) return fail(FXE_ERR_INVALID_ARGS, "n exceeds the context's max_poses");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(FXE_ERR_NO_DEVICE, "cudaSetDevice");
    fxe::launch_build(ctx->S, ctx->W, n, d_genes, nullptr, ctx->stream);
    FXE_TRY(cudaGetLastError(), "autotune launch");
    ++ctx->launches;
    return tune_contacts(ctx, n, reps, ms2, staged);
}

extern "C" fxe_status fxe_context_autotune_sweep(fxe_context* ctx, int32_t n, const int32_t* d_genes, int32_t reps,
                                                 int32_t* caps, double* ms, int32_t max_out, int32_t* n_out) {
    return autotune_sweep(ctx, n, d_genes, reps, caps, ms, max_out, n_out, nullptr, nullptr);
}

extern "C" fxe_status fxe_autotune_lookup(int32_t precision, int32_t scored_atoms, int64_t poses, int32_t* blocks_per_sm) {
    g_err.clear();
    if (!blocks_per_sm || (precision != FXE_PRECISION_REFERENCE && precision != FXE_PRECISION_FAST))
        return fail(FXE_ERR_INVALID_ARGS, "invalid arguments");
    *blocks_per_sm = tuned_blocks(precision, scored_atoms, poses);
    return FXE_OK;
}
