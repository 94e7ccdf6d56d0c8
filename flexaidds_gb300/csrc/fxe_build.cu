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
#include "fxe_common.cuh"

namespace fxe {

constexpr int kBuildWarps = 4;

struct BuildShared {
    float ic[kMaxLig][3];
    float pos[kMaxLig][3];
    int cell[kMaxLig];          // per mobile atom
    float sc[kMaxSc][4];        // side-chain atoms: x, y, z, radius
    int rot[kMaxFlex];          // rotamer of each flexible residue
    double icv[64];
    int gbin[64];     // bin of each gene's value (its entry in the trigonometry tables)
    int gi;           // grid index of the pose
    int bad;
};

// cos and sin of a build angle: the C library's values tabulated by the host for the angles the
// genes produce (so that coordinates match the reference built on the same host bit for bit),
// else the correctly rounded values.
__device__ __forceinline__ void build_trig(const DevSystem& S, const BuildShared& sh, int l, int c, float x,
                                           float* cs, float* sn) {
    const int k = 2 * l + c, src = S.trig_src[k];
    float4 e = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    bool have = false;
    if (src == -2) {
        if ((unsigned)sh.gi < (unsigned)S.n_grid) {
            e = c == 0 ? S.grid_trig_a[sh.gi] : S.grid_trig_d[sh.gi];
            have = true;
        }
    } else {
        const int idx = src < 0 ? 0 : (src < 64 ? sh.gbin[src] : -1);
        if (idx >= 0 && idx < S.trig_cnt[k]) {
            e = S.trig_tab[S.trig_off[k] + idx];
            have = true;
        }
    }
    if (have && __float_as_int(e.x) == __float_as_int(x)) {
        *cs = e.y;
        *sn = e.z;
    } else {
        *cs = (float)cos((double)x);
        *sn = (float)sin((double)x);
    }
}

__device__ __forceinline__ void build_pose(const DevSystem& S, const DevWork& W, int p,
                                           const int32_t* __restrict__ genes,
                                           const double* __restrict__ ic_in, BuildShared& sh,
                                           int lane) {
    const int ng = S.n_genes, nl = S.n_lig;

    // 1. decode + clamp
    for (int g = lane; g < ng; g += 32) {
        double v;
        if (genes) {
            const double u = genes[(size_t)p * ng + g] / (2147483647.0 + 1.0);
            int lo = S.dec_off[g], hi = S.dec_off[g + 1];
            const int base = lo;
            while (lo < hi) {  // first entry >= u
                const int mid = (lo + hi) >> 1;
                if (S.dec_tab[mid] < u) lo = mid + 1; else hi = mid;
            }
            v = S.gene_min[g] + S.gene_del[g] * (double)(lo - base);
            if (g < 64) sh.gbin[g] = lo - base;
        } else {
            v = ic_in[(size_t)p * ng + g];
            // the bin this value would come from; the table entry is used only if its angle matches
            const double b = (v - S.gene_min[g]) / S.gene_del[g];
            if (g < 64) sh.gbin[g] = (b >= 0.0 && b < 2147483647.0) ? (int)rint(b) : -1;
        }
        if (v > S.gene_max[g]) v = S.gene_max[g];
        else if (v < S.gene_min[g]) v = S.gene_min[g];
        W.ic[(size_t)p * ng + g] = v;
        if (g < 64) sh.icv[g] = v;
    }
    for (int l = lane; l < nl; l += 32) {
        const float4 b = S.lig_ic[l];
        sh.ic[l][0] = b.x;
        sh.ic[l][1] = b.y;
        sh.ic[l][2] = b.z;
    }
    if (lane == 0) {
        sh.bad = 0;
        sh.gi = -1;
    }
    if (lane < kMaxFlex) sh.rot[lane] = 0;
    __syncwarp();

    if (lane == 0) {
        // 2. IC assignment, genes in order
        for (int g = 0; g < ng; ++g) {
            const double v = g < 64 ? sh.icv[g] : W.ic[(size_t)p * ng + g];
            const int atm = S.gene_atom[g];
            switch (S.gene_type[g]) {
            case -1: {
                const unsigned gi = (unsigned)v;
                if (gi >= (unsigned)S.n_grid) { sh.bad = 1; break; }
                sh.gi = (int)gi;
                const float4 c = S.grid_ic[gi];
                sh.ic[atm][0] = c.x;
                sh.ic[atm][1] = c.y;
                sh.ic[atm][2] = c.z;
                break;
            }
            case 0: sh.ic[atm][0] = (float)v; break;
            case 1: sh.ic[atm][1] = (float)v; break;
            case 2: {
                sh.ic[atm][2] = (float)v;
                int j = atm, cat = S.lig_rec[atm].w, guard = 0;
                if (cat >= 0) {
                    while (cat != atm && guard++ <= nl) {
                        sh.ic[cat][2] = sh.ic[j][2] + S.lig_shift[cat];
                        j = cat;
                        cat = S.lig_rec[j].w;
                    }
                }
                break;
            }
            case 4: {
                const unsigned r = (unsigned)(v + 0.5);
                if (atm >= 0 && atm < S.n_flex) sh.rot[atm] = (int)r;
                break;
            }
            default: break;
            }
        }
        // 3. buildcc over the rebuild list
        const float* ori = S.ori;
        for (int an = 0; an < S.n_build; ++an) {
            const int l = S.build_order[an];
            const int4 r = S.lig_rec[l];
            const int ref[3] = {r.x, r.y, r.z};
            float x[4], y[4], z[4];
            for (int i = 1; i <= 3; ++i) {
                const int j = ref[i - 1];
                if (j >= 0) {
                    x[i] = sh.pos[j][0];
                    y[i] = sh.pos[j][1];
                    z[i] = sh.pos[j][2];
                } else if (i == 1) {
                    x[i] = 1.0f + ori[0];
                    y[i] = 0.0f + ori[1];
                    z[i] = 0.0f + ori[2];
                } else if (i == 3) {
                    x[i] = 0.0f + ori[0];
                    y[i] = 1.0f + ori[1];
                    z[i] = 0.0f + ori[2];
                } else {
                    x[i] = 0.0f + ori[0];
                    y[i] = 0.0f + ori[1];
                    z[i] = 0.0f + ori[2];
                }
                x[i] += 1e-10f;
                y[i] += 1e-10f;
                z[i] += 1e-10f;
            }
            float a = y[1] * (z[2] - z[3]) + y[2] * (z[3] - z[1]) + y[3] * (z[1] - z[2]);
            float b = z[1] * (x[2] - x[3]) + z[2] * (x[3] - x[1]) + z[3] * (x[1] - x[2]);
            float c = x[1] * (y[2] - y[3]) + x[2] * (y[3] - y[1]) + x[3] * (y[1] - y[2]);
            float op = sqrtf(a * a + b * b + c * c);
            float cx = a / op, cy = b / op, cz = c / op;
            a = x[2] - x[1];
            b = y[2] - y[1];
            c = z[2] - z[1];
            const float d = 1.0f / sqrtf(a * a + b * b + c * c);
            op = sh.ic[l][0] * d;
            const float xn = a * op, yn = b * op, zn = c * op;
            a = cx * cx;
            b = cy * cy;
            c = cz * cz;
            const float angPI = (float)(sh.ic[l][1] * kPi / 180.0f);
            float ct, st;
            build_trig(S, sh, l, 0, angPI, &ct, &st);
            st = -st;
            op = 1.0f - ct;
            const float xk = (cx * cz * op - cy * st) * zn + ((1.0f - a) * ct + a) * xn + (cx * cy * op + cz * st) * yn;
            const float yk = (cy * cx * op - cz * st) * xn + ((1.0f - b) * ct + b) * yn + (cy * cz * op + cx * st) * zn;
            const float zk = (cz * cy * op - cx * st) * yn + ((1.0f - c) * ct + c) * zn + (cz * cx * op + cy * st) * xn;
            const float dihPI = (float)(sh.ic[l][2] * kPi / 180.0f);
            build_trig(S, sh, l, 1, dihPI, &ct, &st);
            op = 1.0f - ct;
            cx = (x[2] - x[1]) * d;
            cy = (y[2] - y[1]) * d;
            cz = (z[2] - z[1]) * d;
            a = cx * cx;
            b = cy * cy;
            c = cz * cz;
            sh.pos[l][0] = (cx * cz * op - cy * st) * zk + ((1.0f - a) * ct + a) * xk + (cx * cy * op + cz * st) * yk + x[1];
            sh.pos[l][1] = (cy * cx * op - cz * st) * xk + ((1.0f - b) * ct + b) * yk + (cy * cz * op + cx * st) * zk + y[1];
            sh.pos[l][2] = (cz * cy * op - cx * st) * yk + ((1.0f - c) * ct + c) * zk + (cz * cx * op + cy * st) * xk + z[1];
        }
    }
    __syncwarp();

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

}  // namespace fxe
