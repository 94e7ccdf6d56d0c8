// fxe_contacts.cu — contact candidates of every (pose, mobile atom).
//
// contacts_kernel, one warp per (pose, mobile atom): the 27-cell scan of get_contlist4
// (LIB/Vcontacts.cpp:1725-1839) over the receptor's cell list of rigid atoms and the pose's
// mobile atoms (side-chain and ligand atoms). The 27 cells' rigid entries are scanned as one
// flat list, 32 at a time, the mobile atoms once; the passing candidates are then sorted into
// the reference's candidate order (cells in scan order, atoms in Calc order within a cell),
// with the reference's single-precision squared distance and its double-precision cut-off test,
// plus the atom's share of the clash pre-filter (LIB/Vcontacts.cpp:36-51): rigid partners and
// the mobile partners processed after it in Calclist order, pairs of one residue within bloops
// bonds left out.
//
// Two forms of the rigid scan, chosen per launch (the autotuner's choice for the size class, or
// the context's setting): the entries read in place from the cell list (global memory, through
// L1 and L2), or staged first in shared memory by bulk copies (cp.async.bulk, one per contiguous
// row of three cells, completing on an mbarrier). Results are the same.
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
// Per-warp staging of an atom's passing candidates, sorted into the reference's order after the
// scan: by (cell in scan order, Calc index), packed into one key.
struct ContactStage {
    int key[128];
    int idx[128];
    float d2[128];
    int coff[28];   // running candidate counts of the 27 cells
    int cst[27];    // their first entries in the cell list
};

// The 27 cells' rigid entries staged in shared memory: scan position 3r + k of the flat list is
// cell k of row r (r = 0..8 over the two slower axes, k over the fastest), and the three cells of
// a row are neighbours in the cell list too, so each row is one contiguous run of entries, moved
// by one bulk copy (positions: 16-byte entries in place at the row's first scan position; Calc
// indices: the run widened to 16-byte boundaries, its entry t at abase[r] + t).
constexpr int kStageCap = 256;                 // entries staged per atom; more: read in place
constexpr int kStageAtoms = kStageCap + 9 * 8;
constexpr long long kStageSpin = 1ll << 22;    // bounded wait for the copies
struct __align__(16) RigidStage {
    float4 pos[kStageCap];
    int atom[kStageAtoms];
    int abase[9];
    unsigned long long bar;
};

__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void bulk_to_shared(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool bar_try_wait(unsigned long long* bar, unsigned phase) {
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(ok) : "r"(smem_addr(bar)), "r"(phase) : "memory");
    return ok != 0;
}
// Waits, at most kStageSpin polls, for the copies of phase 0 of the warp's barrier.
__device__ __forceinline__ bool stage_wait(unsigned long long* bar) {
    bool ok = false;
    for (long long it = 0; it < kStageSpin && !ok; ++it) ok = bar_try_wait(bar, 0u);
    return __all_sync(0xffffffffu, ok);
}

// kStaged: the rigid entries are read from shared memory after bulk copies (rs), else in place.
template <bool kStaged>
__device__ __forceinline__ void contacts_atom(const DevSystem& S, const DevWork& W, int p, int a, int lane,
                                              ContactStage& cs, RigidStage* rs) {
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
    const int n_calc = S.n_rec + S.n_lig;   // keys: cell * n_calc + Calc index
    // scan position 0..26 of linear cell c around box0 (the reference's 27 offsets, which wrap
    // around the rows of the linear index at the grid's faces), or -1
    auto scan_pos = [&](int c) -> int {
        const int o = c - box0 + dim2 + dim + 1;
        if (o < 0) return -1;
        const int di = o / dim2, rem = o - di * dim2, dj = rem / dim, dk = rem - dj * dim;
        return (di <= 2 && dj <= 2 && dk <= 2) ? di * 9 + dj * 3 + dk : -1;
    };
    int nc = 0;
    double clash = 0.0;
    const double permea = (double)S.permeability;
    const float permea_f = S.permeability;
    auto consider = [&](bool in, int pos, int j, float4 pj) {
        bool pass = false;
        float sq = 0.0f;
        if (in) {
            const float dx = __fsub_rn(me.x, pj.x), dy = __fsub_rn(me.y, pj.y), dz = __fsub_rn(me.z, pj.z);
            sq = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            const float nd = __fadd_rn(__fadd_rn(rado, pj.w), kRw);
            // the reference's test sq < nd * nd in double, where the product is exact: the sign of
            // sq - nd * nd rounded once (a fused multiply-add) is the sign of the exact difference
            pass = __fmaf_rn(-nd, nd, sq) < 0.0f && sq != 0.0f;
        }
        const unsigned m = __ballot_sync(kFull, pass);
        if (pass) {
            const int w = nc + __popc(m & lanemask_lt());
            if (w < kMaxCand) {
                cs.key[w] = pos * n_calc + j;
                cs.idx[w] = j;
                cs.d2[w] = sq;
            }
            // clash pre-filter share: rigid partners, and mobile partners processed later
            const int mj = mobile_of(S, j);
            const bool later = mj < 0 || W.mob_rank[lb + mj] > my_rank;
            const float rABf = __fadd_rn(me.w, pj.w);
            const float cdf = permea_f * rABf;
            // surely beyond the clash distance (single-precision bound well outside rounding)
            const bool far = sq > cdf * cdf * 1.0001f;
            if (later && !far) {
                const double rAB = (double)rABf;
                const double cd = permea * rAB;
                const double dist = sqrt((double)sq);
                if (dist < cd && residue_pair(S, a, j) != 1) {
                    // pow(x, -12) as 1 / (x^6)^2: within a few units in the last place of the C
                    // library's pow (which the reference calls) and a tenth of the work
                    const double d2 = dist * dist, d6 = d2 * d2 * d2;
                    const double c2 = cd * cd, c6 = c2 * c2 * c2;
                    clash += (double)kKwall * (1.0 / (d6 * d6) - 1.0 / (c6 * c6));
                }
            }
        }
        nc += __popc(m);
    };
    if (!pg.x) {
        // the rigid atoms of the 27 cells as one list: lane i < 27 counts cell i's entries
        int cnt = 0, st = 0;
        if (lane < 27) {
            const int bi = box0 + dim2 * ((lane / 9) - 1) + dim * (((lane / 3) % 3) - 1) + (lane % 3) - 1;
            if (bi >= 0 && bi < dim3) {
                st = S.cell_start[bi];
                cnt = S.cell_start[bi + 1] - st;
            }
        }
        int inc = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(kFull, inc, o);
            if (lane >= o) inc += v;
        }
        const int total = __shfl_sync(kFull, inc, 31);
        if (lane < 27) {
            cs.coff[lane + 1] = inc;
            cs.cst[lane] = st;
        }
        if (lane == 0) cs.coff[0] = 0;
        __syncwarp();
        // stage the nine rows' entries when they fit
        const bool staged = kStaged && total > 0 && total <= kStageCap;
        bool ready = false;
        if constexpr (kStaged) if (staged) {
            int n_r = 0, st_r = 0, lo4 = 0, len4 = 0;
            if (lane < 9) {
                n_r = cs.coff[3 * lane + 3] - cs.coff[3 * lane];
                const int bi = box0 + dim2 * ((lane / 3) - 1) + dim * ((lane % 3) - 1) - 1;
                const int c0 = bi < 0 ? 0 : bi;
                st_r = c0 < dim3 ? S.cell_start[c0] : 0;
                lo4 = st_r & ~3;
                len4 = n_r > 0 ? ((st_r + n_r + 3) & ~3) - lo4 : 0;
            }
            int aoff = len4;   // exclusive prefix of the widened runs
#pragma unroll
            for (int o = 1; o < 16; o <<= 1) {
                const int v = __shfl_up_sync(kFull, aoff, o);
                if (lane >= o) aoff += v;
            }
            aoff -= len4;
            const int aints = __shfl_sync(kFull, aoff + len4, 8);
            if (lane == 0) {
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(&rs->bar)) : "memory");
                asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                             :: "r"(smem_addr(&rs->bar)), "r"((unsigned)(16 * total + 4 * aints)) : "memory");
            }
            __syncwarp();
            if (lane < 9) {
                rs->abase[lane] = aoff + (st_r - lo4) - cs.coff[3 * lane];
                if (n_r > 0) {
                    bulk_to_shared(&rs->pos[cs.coff[3 * lane]], S.cell_pos + st_r, 16u * n_r, &rs->bar);
                    bulk_to_shared(&rs->atom[aoff], S.cell_atom + lo4, 4u * len4, &rs->bar);
                }
            }
            ready = stage_wait(&rs->bar);
        }
        for (int t0 = 0; t0 < total; t0 += 32) {
            const int t = t0 + lane;
            const bool in = t < total;
            int pos = 0, j = 0;
            float4 pj = make_float4(0, 0, 0, 0);
            if (in) {
                int lo = 0, hi = 26;   // the last cell whose first item is at or before t
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (cs.coff[mid] <= t) lo = mid;
                    else hi = mid - 1;
                }
                pos = lo;
                if (kStaged && ready) {
                    j = rs->atom[rs->abase[lo / 3] + t];
                    pj = rs->pos[t];
                } else {
                    const int k = cs.cst[lo] + (t - cs.coff[lo]);
                    j = S.cell_atom[k];
                    pj = S.cell_pos[k];
                }
            }
            consider(in, pos, j, pj);
        }
        if constexpr (kStaged) if (staged) {
            // the copies are done before the barrier is retired (a second bounded wait when the
            // first gave up)
            if (!ready) ready = stage_wait(&rs->bar);
            if (ready && lane == 0)
                asm volatile("mbarrier.inval.shared::cta.b64 [%0];" :: "r"(smem_addr(&rs->bar)) : "memory");
            __syncwarp();
        }
    } else {
        // a grid re-derived for this pose: every rigid atom, binned on that grid
        const float4 gm = W.pose_gmin[p];
        for (int k0 = 0; k0 < S.n_rec; k0 += 32) {
            const int k = k0 + lane;
            bool in = false;
            int pos = -1;
            float4 pj = make_float4(0, 0, 0, 0);
            if (k < S.n_rec && (nsc == 0 || S.rec_mob[k] < 0)) {
                pj = S.rec_pos[k];
                const int c = (int)((pj.x - gm.x) / kCell) * dim2 + (int)((pj.y - gm.y) / kCell) * dim +
                              (int)((pj.z - gm.z) / kCell);
                pos = scan_pos(c);
                in = pos >= 0;
            }
            consider(in, pos, k, pj);
        }
    }
    // the mobile atoms (side-chain atoms and the ligand) in the 27 cells
#pragma unroll
    for (int s = 0; s < kMaxLig / 32; ++s) {
        if (32 * s >= nm) break;
        const int m = lane + 32 * s;
        int pos = -1;
        float4 pj = make_float4(0, 0, 0, 0);
        if (m < nm) {
            pj = W.mob_pos[lb + m];
            pos = scan_pos(W.mob_cell[lb + m]);
        }
        consider(pos >= 0, pos, m < nm ? slot_of(S, m) : 0, pj);
    }
    if (__any_sync(kFull, clash != 0.0)) clash = warp_sum_d(clash);
    // into the reference's order: bitonic sort of the staged keys
    if (nc <= kMaxCand) {
        int len = 32;
        while (len < nc) len <<= 1;
        for (int i = nc + lane; i < len; i += 32) cs.key[i] = 0x7FFFFFFF;
        __syncwarp();
        for (int k = 2; k <= len; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = lane; i < len; i += 32) {
                    const int l = i ^ j;
                    if (l > i) {
                        const bool up = (i & k) == 0;
                        const int ka = cs.key[i], kb = cs.key[l];
                        if ((ka > kb) == up) {
                            cs.key[i] = kb;
                            cs.key[l] = ka;
                            const int ti = cs.idx[i];
                            cs.idx[i] = cs.idx[l];
                            cs.idx[l] = ti;
                            const float td = cs.d2[i];
                            cs.d2[i] = cs.d2[l];
                            cs.d2[l] = td;
                        }
                    }
                }
                __syncwarp();
            }
        for (int i = lane; i < nc; i += 32) {
            W.cand_idx[cb + i] = cs.idx[i];
            W.cand_d2[cb + i] = cs.d2[i];
        }
    }
    if (lane == 0) {
        W.cand_n[lb + a] = nc > kMaxCand ? -nc : nc;
        W.clash_part[lb + a] = clash;
    }
}

template <bool kStaged>
__global__ void __launch_bounds__(128)
contacts_kernel(DevSystem S, DevWork W, int n) {
    __shared__ ContactStage stage[4];
    RigidStage* rs = nullptr;
    if constexpr (kStaged) {   // (the in-place form allocates no staging)
        __shared__ RigidStage rstage[4];
        rs = &rstage[threadIdx.x >> 5];
    }
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nm = n_mobile(S);
    if (gw >= n * nm) return;
    contacts_atom<kStaged>(S, W, gw / nm, gw % nm, threadIdx.x & 31, stage[threadIdx.x >> 5], rs);
}

// The same over the (pose, mobile atom) items of several jobs.
template <bool kStaged>
__global__ void __launch_bounds__(128)
contacts_kernel_jobs(const Job* __restrict__ jobs, int n_jobs, long long total) {
    __shared__ Job job_all[4];
    __shared__ ContactStage stage[4];
    RigidStage* rs = nullptr;
    if constexpr (kStaged) {
        __shared__ RigidStage rstage[4];
        rs = &rstage[threadIdx.x >> 5];
    }
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (gw >= total) return;
    const int j = find_job(jobs, n_jobs, gw, true);
    Job& job = job_all[wib];
    copy_job(&job, &jobs[j], lane);
    const int nm = n_mobile(job.S);
    const long long r = gw - job.warp0;
    contacts_atom<kStaged>(job.S, job.W, (int)(r / nm), (int)(r % nm), lane, stage[wib], rs);
}

// The order pose_kernel takes the poses in: the poses with the most scored atoms first, among
// them the costliest first (sum over the pose's atoms of the squared candidate count, which the
// hull walk's plane tests grow with), so that the slowest poses start early and the launch does
// not end on one of them while the SMs run dry, and the poses a lockstep block steps through
// together have as many atoms; then the
// poses that need no polyhedra (the clash pre-filter rejects them, or they left the grid), so
// that the warps of a block, which step through the atoms together, are not held by poses that
// have nothing to do. Sorted in segments of kOrderSeg poses, one block each. The order changes
// no result.
// A launch of lockstep blocks takes tiles of `tile` neighbouring queue entries; its first `deal`
// tiles (as many full tiles as the device runs at once) start together. When they are all the
// launch has, or when its scored poses do not fill them, the launch lasts about as long as its
// slowest first tile: there the sorted poses are dealt round-robin over those tiles (tile t gets
// sorted entries t, t + deal, ...), so each holds one of the costliest poses and the scored poses
// spread over every SM, the rejected ones taking the tiles' last slots and the later tiles.
// Otherwise (the scored poses fill more than the first tiles) the sorted order stands.
constexpr int kOrderSeg = 4096;

// Queue position of sorted entry i of a segment.
__device__ __forceinline__ int dealt_position(int i, int deal, int tile) {
    return deal > 0 && i < deal * tile ? (i % deal) * tile + i / deal : i;
}

// Whether a sorted single segment of m poses, n_scored of them scored, is dealt over `deal` tiles.
__device__ __forceinline__ int deal_tiles(int m, int n_scored, int deal, int tile) {
    return deal > 0 && (deal == m / tile || n_scored < deal * tile) ? deal : 0;
}

// The sort key of pose p: minus its cost, or 1 for a pose the polyhedron launch rejects at once.
__device__ __forceinline__ long long pose_order_key(const DevWork& W, int nm, int p) {
    if (W.pose_grid[p].z) return 1;
    const int* cn = W.cand_n + (size_t)p * nm;
    const double* cp = W.clash_part + (size_t)p * nm;
    long long cost = 0;
    double clash = 0.0;
    for (int a = 0; a < nm; ++a) {
        const int k = cn[a];
        if (k > 0) cost += (long long)k * k;
        clash += cp[a];
    }
    // (the launch's own test sums the same terms in another order: a pose within rounding of the
    // threshold may be placed on the other side, which only moves it in the queue)
    if (clash >= kClashThreshold) return 1;
    // scored poses with more atoms first (a lockstep block steps through as many atoms as its
    // largest pose has), then the costliest
    return -(((long long)nm << 40) | cost);
}

__global__ void __launch_bounds__(1024) order_poses_kernel(DevWork W, int nm, int n, int* __restrict__ order, int deal,
                                                           int tile) {
    __shared__ long long key[kOrderSeg];
    __shared__ int idx[kOrderSeg];
    __shared__ int n_scored;
    if (threadIdx.x == 0) n_scored = 0;
    const int base = blockIdx.x * kOrderSeg;
    const int m = min(kOrderSeg, n - base);
    int len = 1;
    while (len < m) len <<= 1;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
        long long c = 0x7FFFFFFFFFFFFFFFll;   // padding sorts last
        if (i < m) c = pose_order_key(W, nm, base + i);
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
    // the scored poses (keys <= 0) of the segment
    int c = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) c += key[i] <= 0;
    if (c) atomicAdd(&n_scored, c);
    __syncthreads();
    const int dl = deal_tiles(m, n_scored, deal, tile);
    for (int i = threadIdx.x; i < m; i += blockDim.x) order[base + dealt_position(i, dl, tile)] = base + idx[i];
}

// The same over the poses of several jobs (global pose index gp of the launch).
__global__ void __launch_bounds__(1024) order_poses_jobs_kernel(const Job* __restrict__ jobs, int n_jobs, int n,
                                                                int* __restrict__ order, int deal, int tile) {
    __shared__ long long key[kOrderSeg];
    __shared__ int idx[kOrderSeg];
    __shared__ int n_scored;
    if (threadIdx.x == 0) n_scored = 0;
    const int base = blockIdx.x * kOrderSeg;
    const int m = min(kOrderSeg, n - base);
    int len = 1;
    while (len < m) len <<= 1;
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
        long long c = 0x7FFFFFFFFFFFFFFFll;
        if (i < m) {
            const int gp = base + i;
            const Job& J = jobs[find_job(jobs, n_jobs, gp, false)];
            c = pose_order_key(J.W, J.S.n_sc + J.S.n_lig, gp - J.pose0);
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
    // the scored poses (keys <= 0) of the segment
    int c = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) c += key[i] <= 0;
    if (c) atomicAdd(&n_scored, c);
    __syncthreads();
    const int dl = deal_tiles(m, n_scored, deal, tile);
    for (int i = threadIdx.x; i < m; i += blockDim.x) order[base + dealt_position(i, dl, tile)] = base + idx[i];
}

// deal: full tiles to deal the sorted poses over (one segment only; 0 keeps the sorted order);
// tile: poses per tile.
void launch_order_poses_jobs(const Job* jobs, int n_jobs, int total, int* order, cudaStream_t st, int deal,
                             int tile) {
    if (total > kOrderSeg || tile < 1) deal = 0;
    order_poses_jobs_kernel<<<(total + kOrderSeg - 1) / kOrderSeg, 1024, 0, st>>>(jobs, n_jobs, total, order, deal,
                                                                                  tile);
}

void launch_order_poses(const DevSystem& S, const DevWork& W, int n, cudaStream_t st, int deal, int tile) {
    if (n > kOrderSeg || tile < 1) deal = 0;
    order_poses_kernel<<<(n + kOrderSeg - 1) / kOrderSeg, 1024, 0, st>>>(W, S.n_sc + S.n_lig, n, W.pose_order, deal,
                                                                         tile);
}

void launch_contacts(const DevSystem& S, const DevWork& W, int n, cudaStream_t st, bool staged) {
    const long warps = (long)n * (S.n_sc + S.n_lig);
    const unsigned blocks = (unsigned)((warps + 3) / 4);
    if (staged) contacts_kernel<true><<<blocks, 128, 0, st>>>(S, W, n);
    else contacts_kernel<false><<<blocks, 128, 0, st>>>(S, W, n);
}

void launch_contacts_jobs(const Job* jobs, int n_jobs, long long total_items, cudaStream_t st, bool staged) {
    const unsigned blocks = (unsigned)((total_items + 3) / 4);
    if (staged) contacts_kernel_jobs<true><<<blocks, 128, 0, st>>>(jobs, n_jobs, total_items);
    else contacts_kernel_jobs<false><<<blocks, 128, 0, st>>>(jobs, n_jobs, total_items);
}

}  // namespace fxe
