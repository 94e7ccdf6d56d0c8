// fxe_build.cu — gene decode, IC assignment and pose build, one warp per pose.
//
// Compiled with --fmad=false: the single-precision build arithmetic is evaluated exactly as
// written (no fused multiply-adds), like the reference's buildcc (LIB/buildcc.cpp:6-134).
//
// Per pose:
//   1. genes -> ICs: genetoic (LIB/gaboom.cpp:2887-2906) as a binary search in the running
//      bin totals the host precomputes, then the clamp of eval_chromosome
//      (LIB/gaboom.cpp:1845-1866);
//   2. IC assignment of ic2cf (LIB/ic2cf.cpp:53-105): grid index, angle, dihedral with the
//      rec[3] cascade;
//   3. buildcc over the rebuild list;
//   4. the side-chain atoms of the rotamers the rotamer genes select (LIB/ic2cf.cpp:90-94 and
//      index_protein's refill of the scored Calc slots, LIB/Vcontacts.cpp:1600-1625);
//   5. the cell grid of index_protein for this pose (LIB/Vcontacts.cpp:1584-1645: the
//      receptor's steady grid, re-derived when a mobile atom leaves the receptor's box), the
//      mobile atoms' cells and their position in Calclist order (cell, then Calc index).
#include "fxe_place.cuh"

namespace fxe {

constexpr int kBuildWarps = 4;

__device__ __forceinline__ void build_pose(const DevSystem& S, const DevWork& W, int p,
                                           const int32_t* __restrict__ genes,
                                           const double* __restrict__ ic_in, BuildShared& sh,
                                           int lane) {
    const int nl = S.n_lig;
    double* const ic_row = W.ic + (size_t)p * S.n_genes;

    // 1. decode + clamp
    decode_ics(S, p, genes, ic_in, true, ic_row, sh, lane);
    reset_pose(S, sh, lane);
    __syncwarp();

    // 2-3. IC assignment, genes in order, and buildcc over the rebuild list
    if (lane == 0) assign_ics(S, sh, ic_row);
    __syncwarp();
    build_atoms(S, sh, lane);

    // 4. side-chain atoms of the selected rotamers
    const int nsc = S.n_sc, nm = nsc + nl;
    if (lane < nsc) {
        const int r = S.sc_res[lane];
        const int4 fi = S.flex_info[r];
        const int rot = sh.rot[r];
        const float4 q = S.sc_rot[fi.x + rot * fi.z + (lane - fi.y)];
        sh.sc[lane][0] = q.x;
        sh.sc[lane][1] = q.y;
        sh.sc[lane][2] = q.z;
        sh.sc[lane][3] = q.w;
    }
    __syncwarp();
    auto mpos = [&](int m, int k) -> float { return m < nsc ? sh.sc[m][k] : sh.pos[m - nsc][k]; };

    // 5. cell grid of this pose
    bool below[3] = {false, false, false}, above[3] = {false, false, false};
    float mn[3] = {S.gmin[0], S.gmin[1], S.gmin[2]};
    float mx[3] = {S.gmax[0], S.gmax[1], S.gmax[2]};
    for (int m = lane; m < nm; m += 32)
        for (int k = 0; k < 3; ++k) {
            const float v = mpos(m, k);
            if (v < mn[k]) { mn[k] = v; below[k] = true; }
            else if (v > mx[k]) { mx[k] = v; above[k] = true; }
        }
    bool alter = false;
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
        alter |= __any_sync(0xffffffffu, below[k] || above[k]);
    }
    float gmin[3];
    int dim;
    if (alter) {
        float mw = S.maxwidth;
        for (int k = 0; k < 3; ++k) {
            gmin[k] = mn[k] < 0.0f ? (float)((int)mn[k] - 1.0) : (float)((int)mn[k] + 1.0);
            const float gmx = mx[k] < 0.0f ? (float)((int)mx[k] - 1.0) : (float)((int)mx[k] + 1.0);
            const float diff = gmx - gmin[k];
            if (diff > mw) mw = diff;
        }
        dim = (int)(mw / kCell) + 1;
    } else {
        gmin[0] = S.gmin[0];
        gmin[1] = S.gmin[1];
        gmin[2] = S.gmin[2];
        dim = S.dim;
    }
    const int dim2 = dim * dim, dim3 = dim2 * dim;
    for (int m = lane; m < nm; m += 32) {
        const int bi = (int)((mpos(m, 0) - gmin[0]) / kCell) * dim2 + (int)((mpos(m, 1) - gmin[1]) / kCell) * dim +
                       (int)((mpos(m, 2) - gmin[2]) / kCell);
        if (bi < 0 || bi >= dim3) sh.bad = 2;
        sh.cell[m] = bi;
    }
    __syncwarp();
    const size_t base = (size_t)p * nm;
    for (int m = lane; m < nm; m += 32) {
        const int c = sh.cell[m];
        int rank = 0;
        for (int q = 0; q < nm; ++q) {
            const int cq = sh.cell[q];
            rank += (cq < c) || (cq == c && q < m);
        }
        const float rad = m < nsc ? sh.sc[m][3] : S.lig_radius[m - nsc];
        W.mob_pos[base + m] = make_float4(mpos(m, 0), mpos(m, 1), mpos(m, 2), rad);
        W.mob_cell[base + m] = c;
        W.mob_rank[base + m] = rank;
    }
    if (lane == 0) {
        W.pose_grid[p] = make_int4(alter ? 1 : 0, dim, sh.bad, 0);
        W.pose_gmin[p] = make_float4(gmin[0], gmin[1], gmin[2], 0.0f);
    }
}

__global__ void __launch_bounds__(kBuildWarps * 32)
build_kernel(DevSystem S, DevWork W, int n, const int32_t* __restrict__ genes,
             const double* __restrict__ ic_in) {
    __shared__ BuildShared sh_all[kBuildWarps];
    const int wib = threadIdx.x >> 5;
    const int p = blockIdx.x * kBuildWarps + wib;
    if (p >= n) return;
    build_pose(S, W, p, genes, ic_in, sh_all[wib], threadIdx.x & 31);
}

// The same over the poses of several jobs: the warp finds its job, takes the job's system and
// workspace into shared memory and builds its pose there.
__global__ void __launch_bounds__(kBuildWarps * 32)
build_kernel_jobs(const Job* __restrict__ jobs, int n_jobs, int total) {
    __shared__ BuildShared sh_all[kBuildWarps];
    __shared__ Job job_all[kBuildWarps];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gp = blockIdx.x * kBuildWarps + wib;
    if (gp >= total) return;
    const int j = find_job(jobs, n_jobs, gp, false);
    Job& job = job_all[wib];
    copy_job(&job, &jobs[j], lane);
    build_pose(job.S, job.W, gp - job.pose0, job.genes, nullptr, sh_all[wib], lane);
}

void launch_build(const DevSystem& S, const DevWork& W, int n, const int32_t* genes,
                  const double* ic, cudaStream_t st) {
    const int blocks = (n + kBuildWarps - 1) / kBuildWarps;
    build_kernel<<<blocks, kBuildWarps * 32, 0, st>>>(S, W, n, genes, ic);
}

void launch_build_jobs(const Job* jobs, int n_jobs, int total, cudaStream_t st) {
    const int blocks = (total + kBuildWarps - 1) / kBuildWarps;
    build_kernel_jobs<<<blocks, kBuildWarps * 32, 0, st>>>(jobs, n_jobs, total);
}

// Gene decode alone (fxe_decode_genes): genetoic of every gene of n chromosomes, one thread per
// gene, clamped into the gene limits as eval_chromosome leaves them when clamp is set.
__global__ void decode_kernel(DevSystem S, long long n, const int32_t* __restrict__ genes, double* __restrict__ ic,
                              int clamp) {
    const long long total = n * S.n_genes;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(t % S.n_genes);
        double v = S.gene_min[g] + S.gene_del[g] * (double)gene_bin(S, g, genes[t]);
        if (clamp) {
            if (v > S.gene_max[g]) v = S.gene_max[g];
            else if (v < S.gene_min[g]) v = S.gene_min[g];
        }
        ic[t] = v;
    }
}

void launch_decode(const DevSystem& S, long long n, const int32_t* genes, double* ic, int clamp, cudaStream_t st) {
    const long long total = n * S.n_genes;
    long long blocks = (total + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    decode_kernel<<<(unsigned)blocks, 256, 0, st>>>(S, n, genes, ic, clamp);
}

}  // namespace fxe
