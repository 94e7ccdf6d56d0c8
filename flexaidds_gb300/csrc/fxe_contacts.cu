// fxe_contacts.cu — contact candidates of every (pose, ligand atom).
//
// contacts_kernel, one warp per (pose, ligand atom): the 27-cell scan of get_contlist4
// (LIB/Vcontacts.cpp:1725-1839) over the receptor's cell list and the pose's ligand atoms, in
// the reference's candidate order (cells in scan order, atoms in Calc order within a cell),
// with the reference's single-precision squared distance and its double-precision cut-off test,
// plus the atom's share of the clash pre-filter (LIB/Vcontacts.cpp:36-51): receptor partners
// and the ligand partners processed after it in Calclist order.
#include "fxe_common.cuh"

namespace fxe {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// ------------------------------------------------------------------------------------------
// contacts_kernel
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void contacts_atom(const DevSystem& S, const DevWork& W, int p, int a, int lane) {
    const int nl = S.n_lig;
    const size_t lb = (size_t)p * nl;
    const int4 pg = W.pose_grid[p];
    const size_t cb = (lb + a) * kMaxCand;
    if (pg.z) {  // the pose left the grid the reference can index
        if (lane == 0) {
            W.cand_n[lb + a] = 0;
            W.clash_part[lb + a] = 0.0;
        }
        return;
    }
    const float4 me = W.lig_pos[lb + a];
    const float rado = me.w + kRw;
    const int my_rank = W.lig_rank[lb + a];
    const int dim = pg.y, dim2 = dim * dim, dim3 = dim2 * dim;
    const int box0 = W.lig_cell[lb + a];
    // ligand atoms held by this lane (atom lane + 32 * slot): cell offset key 0..26 or -1
    int key[kMaxLig / 32];
    float4 lpos[kMaxLig / 32];
#pragma unroll
    for (int s = 0; s < kMaxLig / 32; ++s) {
        const int l = lane + 32 * s;
        key[s] = -1;
        lpos[s] = make_float4(0, 0, 0, 0);
        if (l < nl) {
            lpos[s] = W.lig_pos[lb + l];
            const int o = W.lig_cell[lb + l] - box0 + dim2 + dim + 1;
            if (o >= 0) {
                const int di = o / dim2, rem = o - di * dim2, dj = rem / dim, dk = rem - dj * dim;
                if (di <= 2 && dj <= 2 && dk <= 2) key[s] = di * 9 + dj * 3 + dk;
            }
        }
    }
    const float4 gm = W.pose_gmin[p];
    int nc = 0;
    double clash = 0.0;
    const double permea = (double)S.permeability;
    auto consider = [&](bool in, int j, float4 pj) {
        bool pass = false;
        float sq = 0.0f;
        if (in) {
            const float dx = __fsub_rn(me.x, pj.x), dy = __fsub_rn(me.y, pj.y), dz = __fsub_rn(me.z, pj.z);
            sq = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            const float nd = __fadd_rn(__fadd_rn(rado, pj.w), kRw);
            pass = ((double)sq < (double)nd * (double)nd) && sq != 0.0f;
        }
        const unsigned m = __ballot_sync(kFull, pass);
        if (pass) {
            const int w = nc + __popc(m & lanemask_lt());
            if (w < kMaxCand) {
                W.cand_idx[cb + w] = j;
                W.cand_d2[cb + w] = sq;
            }
            // clash pre-filter share: receptor partners, and ligand partners processed later
            const bool later = j < S.n_rec || W.lig_rank[lb + (j - S.n_rec)] > my_rank;
            if (later) {
                const double rAB = (double)__fadd_rn(me.w, pj.w);
                const double cd = permea * rAB;
                const double dist = sqrt((double)sq);
                if (dist < cd) {
                    const bool intra = j >= S.n_rec;
                    if (!intra || S.bonded[a * nl + (j - S.n_rec)] < 0)
                        clash += (double)kKwall * (pow(dist, -12.0) - pow(cd, -12.0));
                }
            }
        }
        nc += __popc(m);
    };
    for (int i = 0; i < 27; ++i) {
        const int bi = box0 + dim2 * ((i / 9) - 1) + dim * (((i / 3) % 3) - 1) + (i % 3) - 1;
        if (bi < 0 || bi >= dim3) continue;
        if (!pg.x) {
            const int s0 = S.cell_start[bi], s1 = S.cell_start[bi + 1];
            for (int k0 = s0; k0 < s1; k0 += 32) {
                const int k = k0 + lane;
                const bool in = k < s1;
                const int j = in ? S.cell_atom[k] : 0;
                const float4 pj = in ? S.cell_pos[k] : make_float4(0, 0, 0, 0);
                consider(in, j, pj);
            }
        } else {
            // a grid re-derived for this pose: scan every receptor atom for cell bi
            for (int k0 = 0; k0 < S.n_rec; k0 += 32) {
                const int k = k0 + lane;
                bool in = false;
                float4 pj = make_float4(0, 0, 0, 0);
                if (k < S.n_rec) {
                    pj = S.rec_pos[k];
                    const int cb2 = (int)((pj.x - gm.x) / kCell) * dim2 + (int)((pj.y - gm.y) / kCell) * dim +
                                    (int)((pj.z - gm.z) / kCell);
                    in = cb2 == bi;
                }
                consider(in, k, pj);
            }
        }
#pragma unroll
        for (int s = 0; s < kMaxLig / 32; ++s) {
            if (32 * s >= nl) break;
            consider(key[s] == i, S.n_rec + lane + 32 * s, lpos[s]);
        }
    }
    clash = warp_sum_d(clash);
    if (lane == 0) {
        W.cand_n[lb + a] = nc > kMaxCand ? -nc : nc;
        W.clash_part[lb + a] = clash;
    }
}

__global__ void __launch_bounds__(128)
contacts_kernel(DevSystem S, DevWork W, int n) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nl = S.n_lig;
    if (gw >= n * nl) return;
    contacts_atom(S, W, gw / nl, gw % nl, threadIdx.x & 31);
}

// The same over the (pose, ligand atom) items of several jobs.
__global__ void __launch_bounds__(128)
contacts_kernel_jobs(const Job* __restrict__ jobs, int n_jobs, long long total) {
    __shared__ Job job_all[4];
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (gw >= total) return;
    const int j = find_job(jobs, n_jobs, gw, true);
    Job& job = job_all[wib];
    copy_job(&job, &jobs[j], lane);
    const int nl = job.S.n_lig;
    const long long r = gw - job.warp0;
    contacts_atom(job.S, job.W, (int)(r / nl), (int)(r % nl), lane);
}

void launch_contacts(const DevSystem& S, const DevWork& W, int n, cudaStream_t st) {
    const long warps = (long)n * S.n_lig;
    contacts_kernel<<<(unsigned)((warps + 3) / 4), 128, 0, st>>>(S, W, n);
}

void launch_contacts_jobs(const Job* jobs, int n_jobs, long long total_items, cudaStream_t st) {
    contacts_kernel_jobs<<<(unsigned)((total_items + 3) / 4), 128, 0, st>>>(jobs, n_jobs, total_items);
}

}  // namespace fxe
