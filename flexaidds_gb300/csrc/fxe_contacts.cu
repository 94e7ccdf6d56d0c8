// fxe_contacts.cu — contact candidates of every (pose, mobile atom).
//
// contacts_kernel, one warp per (pose, mobile atom): the 27-cell scan of get_contlist4
// (LIB/Vcontacts.cpp:1725-1839) over the receptor's cell list of rigid atoms and the pose's
// mobile atoms (side-chain atoms at their Calc places among the rigid atoms, then the ligand),
// in the reference's candidate order (cells in scan order, atoms in Calc order within a cell),
// with the reference's single-precision squared distance and its double-precision cut-off test,
// plus the atom's share of the clash pre-filter (LIB/Vcontacts.cpp:36-51): rigid partners and
// the mobile partners processed after it in Calclist order, pairs of one residue within bloops
// bonds left out.
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
    const int nsc = S.n_sc, nm = nsc + S.n_lig;
    const size_t lb = (size_t)p * nm;
    const int4 pg = W.pose_grid[p];
    const size_t cb = (lb + a) * kMaxCand;
    if (pg.z) {  // the pose left the grid the reference can index
        if (lane == 0) {
            W.cand_n[lb + a] = 0;
            W.clash_part[lb + a] = 0.0;
        }
        return;
    }
    const float4 me = W.mob_pos[lb + a];
    const float rado = me.w + kRw;
    const int my_rank = W.mob_rank[lb + a];
    const int dim = pg.y, dim2 = dim * dim, dim3 = dim2 * dim;
    const int box0 = W.mob_cell[lb + a];
    // mobile atoms held by this lane (atom lane + 32 * slot): cell offset key 0..26 or -1; the
    // side-chain atoms (fewer than 33) are the lanes of slot 0
    int key[kMaxLig / 32];
    float4 lpos[kMaxLig / 32];
#pragma unroll
    for (int s = 0; s < kMaxLig / 32; ++s) {
        const int m = lane + 32 * s;
        key[s] = -1;
        lpos[s] = make_float4(0, 0, 0, 0);
        if (m < nm) {
            lpos[s] = W.mob_pos[lb + m];
            const int o = W.mob_cell[lb + m] - box0 + dim2 + dim + 1;
            if (o >= 0) {
                const int di = o / dim2, rem = o - di * dim2, dj = rem / dim, dk = rem - dj * dim;
                if (di <= 2 && dj <= 2 && dk <= 2) key[s] = di * 9 + dj * 3 + dk;
            }
        }
    }
    const int my_slot = lane < nsc ? S.sc_slot[lane] : 0;
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
            // clash pre-filter share: rigid partners, and mobile partners processed later
            const int mj = mobile_of(S, j);
            const bool later = mj < 0 || W.mob_rank[lb + mj] > my_rank;
            if (later) {
                const double rAB = (double)__fadd_rn(me.w, pj.w);
                const double cd = permea * rAB;
                const double dist = sqrt((double)sq);
                if (dist < cd && residue_pair(S, a, j) != 1)
                    clash += (double)kKwall * (pow(dist, -12.0) - pow(cd, -12.0));
            }
        }
        nc += __popc(m);
    };
    // rigid atoms of one cell in Calc order, entries [k0, k1) of the cell list (or, on a grid
    // re-derived for this pose, Calc indices [k0, k1) that fall into cell bi)
    auto scan_rigid = [&](int k0, int k1, int bi) {
        for (int kb = k0; kb < k1; kb += 32) {
            const int k = kb + lane;
            bool in = k < k1;
            int j = 0;
            float4 pj = make_float4(0, 0, 0, 0);
            if (!pg.x) {
                if (in) {
                    j = S.cell_atom[k];
                    pj = S.cell_pos[k];
                }
            } else if (in) {
                j = k;
                pj = S.rec_pos[k];
                const int cb2 = (int)((pj.x - gm.x) / kCell) * dim2 + (int)((pj.y - gm.y) / kCell) * dim +
                                (int)((pj.z - gm.z) / kCell);
                in = cb2 == bi && (nsc == 0 || S.rec_mob[k] < 0);
            }
            consider(in, j, pj);
        }
    };
    for (int i = 0; i < 27; ++i) {
        const int bi = box0 + dim2 * ((i / 9) - 1) + dim * (((i / 3) % 3) - 1) + (i % 3) - 1;
        if (bi < 0 || bi >= dim3) continue;
        int k0, k1;
        if (!pg.x) {
            k0 = S.cell_start[bi];
            k1 = S.cell_start[bi + 1];
        } else {
            k0 = 0;
            k1 = S.n_rec;
        }
        // side-chain atoms in this cell take their Calc places among the rigid atoms
        unsigned scm = __ballot_sync(kFull, lane < nsc && key[0] == i);
        while (scm) {
            const int q = __ffs(scm) - 1;
            scm &= scm - 1;
            const int qs = __shfl_sync(kFull, my_slot, q);
            int split = qs;
            if (!pg.x) {   // rigid entries of the cell before Calc index qs
                split = k0;
                for (int kb = k0; kb < k1; kb += 32) {
                    const int k = kb + lane;
                    const unsigned lt = __ballot_sync(kFull, k < k1 && S.cell_atom[k] < qs);
                    split += __popc(lt);
                    if (lt != kFull) break;
                }
            }
            scan_rigid(k0, split, bi);
            consider(lane == q, qs, lpos[0]);
            k0 = split;
        }
        scan_rigid(k0, k1, bi);
#pragma unroll
        for (int s = 0; s < kMaxLig / 32; ++s) {
            if (32 * s >= nm) break;
            const int m = lane + 32 * s;
            consider(key[s] == i && m >= nsc, S.n_rec + (m - nsc), lpos[s]);
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
    const int nm = n_mobile(S);
    if (gw >= n * nm) return;
    contacts_atom(S, W, gw / nm, gw % nm, threadIdx.x & 31);
}

// The same over the (pose, mobile atom) items of several jobs.
__global__ void __launch_bounds__(128)
contacts_kernel_jobs(const Job* __restrict__ jobs, int n_jobs, long long total) {
    __shared__ Job job_all[4];
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (gw >= total) return;
    const int j = find_job(jobs, n_jobs, gw, true);
    Job& job = job_all[wib];
    copy_job(&job, &jobs[j], lane);
    const int nm = n_mobile(job.S);
    const long long r = gw - job.warp0;
    contacts_atom(job.S, job.W, (int)(r / nm), (int)(r % nm), lane);
}

// The order pose_kernel takes the poses in: costliest first (sum over the pose's atoms of the
// squared candidate count, which the hull walk's plane tests grow with), so that the slowest
// poses start early and the launch does not end on one of them while the SMs run dry. Sorted in
// segments of kOrderSeg poses, one block each.
constexpr int kOrderSeg = 4096;

__global__ void __launch_bounds__(1024) order_poses_kernel(const int* __restrict__ cand_n, int nm, int n,
                                                           int* __restrict__ order) {
    __shared__ long long key[kOrderSeg];
    __shared__ int idx[kOrderSeg];
    const int base = blockIdx.x * kOrderSeg;
    const int m = min(kOrderSeg, n - base);
    int len = 1;
    while (len < m) len <<= 1;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
        long long c = 0x7FFFFFFFFFFFFFFFll;   // padding sorts last
        if (i < m) {
            const int* cn = cand_n + (size_t)(base + i) * nm;
            long long cost = 0;
            for (int a = 0; a < nm; ++a) {
                const int k = cn[a];
                if (k > 0) cost += (long long)k * k;
            }
            c = -cost;
        }
        key[i] = c;
        idx[i] = i;
    }
    __syncthreads();
    for (int k = 2; k <= len; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < len; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    const long long a = key[i], b = key[l];
                    const bool gt = a > b || (a == b && idx[i] > idx[l]);
                    if (gt == up) {
                        key[i] = b;
                        key[l] = a;
                        const int t = idx[i];
                        idx[i] = idx[l];
                        idx[l] = t;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < m; i += blockDim.x) order[base + i] = base + idx[i];
}

void launch_order_poses(const DevSystem& S, const DevWork& W, int n, cudaStream_t st) {
    order_poses_kernel<<<(n + kOrderSeg - 1) / kOrderSeg, 1024, 0, st>>>(W.cand_n, S.n_sc + S.n_lig, n, W.pose_order);
}

void launch_contacts(const DevSystem& S, const DevWork& W, int n, cudaStream_t st) {
    const long warps = (long)n * (S.n_sc + S.n_lig);
    contacts_kernel<<<(unsigned)((warps + 3) / 4), 128, 0, st>>>(S, W, n);
}

void launch_contacts_jobs(const Job* jobs, int n_jobs, long long total_items, cudaStream_t st) {
    contacts_kernel_jobs<<<(unsigned)((total_items + 3) / 4), 128, 0, st>>>(jobs, n_jobs, total_items);
}

}  // namespace fxe
