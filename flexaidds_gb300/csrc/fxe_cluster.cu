// fxe_cluster.cu — CF-based clustering of a docking result on the device: cluster
// (LIB/cluster.cpp:9-182), the reference's default clustering of the GA's ensemble
// (LIB/top.cpp:1351-1354).
//
// The reference builds the ligand of every chromosome once into a coordinate cache
// (calc_rmsd_chrom, LIB/calc_rmsd_chrom.cpp:7-145; LIB/cluster.cpp:94-113), then forms clusters
// one at a time: the first chromosome no cluster holds yet heads the next cluster and takes in
// every later unclustered chromosome whose ligand RMSD to it is at most FA->cluster_rmsd
// (LIB/cluster.cpp:116-175), until every chromosome is clustered or max_results clusters exist.
//
// Here: one kernel builds every ligand (the pose build's placement arithmetic), stored by coordinate
// (x of atom 0 for all chromosomes, then y, ...) so that each pass reads whole sectors; one
// launch per cluster compares the unclustered chromosomes with the head and leaves the next
// head (the first chromosome it did not take) for the next launch, so the passes run back to back
// with no host round trip; a last one-block kernel adds up each cluster's terms and the RMSD
// between cluster heads. Compiled with --fmad=false: the RMSD sums are evaluated exactly as the
// reference writes them (no fused multiply-adds).
#include "fxe_place.cuh"

namespace fxe {

// Ligand of each chromosome from its ICs, one thread per chromosome and kThreadBuild chromosomes
// per block: the IC assignment of calc_rmsd_chrom (the same as ic2cf's) and buildcc, the ligand
// atoms in order, stored as xyz[(3 * l + c) * n + p]. A warp builds 32 ligands in step, so the
// serial chain of each atom costs one instruction stream for 32 chromosomes. calc_rmsd_chrom uses
// to_ic as stored, without eval_chromosome's clamp (the host admits only ICs within their gene
// limits, so the two agree). Each thread forms its atoms' ICs without replaying the assignment:
// the host's replay names the gene (or grid point, or base IC) that sets each distance, angle and
// dihedral last, and the atoms whose shifts a dihedral cascade adds (dis_src, trig_src, cas_*).
// Shared memory, per block: the placed atoms [3 * n_lig][kThreadBuild], and per gene its value as
// a float and its bin [n_genes][kThreadBuild] each.
constexpr int kThreadBuild = 64;
constexpr int kPassThreads = 256;

size_t thread_build_smem(const DevSystem& S) {
    return sizeof(float) * kThreadBuild * (3 * (size_t)S.n_lig + 2 * (size_t)S.n_genes);
}

__global__ void __launch_bounds__(kThreadBuild)
cluster_build_thread_kernel(DevSystem S, int n, const double* __restrict__ ic, float* __restrict__ xyz,
                            int* __restrict__ bad) {
    extern __shared__ __align__(16) float tsm[];
    const int t = threadIdx.x, ng = S.n_genes, nl = S.n_lig;
    float* pos = tsm;                                    // [(3 l + k) * kThreadBuild + t]
    float* fv = pos + (size_t)3 * nl * kThreadBuild;     // [g * kThreadBuild + t]
    int* gb = reinterpret_cast<int*>(fv + (size_t)ng * kThreadBuild);
    const int p = blockIdx.x * kThreadBuild + t;
    if (p >= n) return;   // no block-wide barrier follows
    const double* row = ic + (size_t)p * ng;
    int gi = -1, st = 0;
    for (int g = 0; g < ng; ++g) {
        const double v = row[g];
        if (!(v >= S.gene_min[g] && v <= S.gene_max[g])) st |= 2;
        // a guess, in single precision, of the bin this value comes from; a table entry is used
        // only if its angle matches, and a miss retries with the bin formed in double precision
        const float f = (float)v;
        const float b = (f - S.gene_minf[g]) * S.gene_idelf[g];
        gb[g * kThreadBuild + t] = (b >= 0.0f && b < 2.0e9f) ? (int)rintf(b) : -1;
        fv[g * kThreadBuild + t] = f;
        if (S.gene_type[g] == -1) {
            // the grid gene (LIB/ic2cf.cpp:60-67); an index past the grid is an error and leaves
            // the anchor's base ICs
            const unsigned u = (unsigned)v;
            if (u >= (unsigned)S.n_grid) st |= 1;
            else gi = (int)u;
        }
    }
    if (st) atomicOr(bad, st);
    for (int k = 0; k < 3 * nl; ++k) pos[k * kThreadBuild + t] = 0.0f;
    const float4 grid = gi >= 0 ? S.grid_ic[gi] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int an = 0; an < S.n_build; ++an) {
        const int l = S.build_order[an];
        const float4 base = S.lig_ic[l];
        // distance, angle and dihedral as the IC assignment leaves them
        const int sd = S.dis_src[l], sa = S.trig_src[2 * l], sx = S.trig_src[2 * l + 1];
        const float dis = sd == -2 ? (gi >= 0 ? grid.x : base.x) : (sd >= 0 ? fv[sd * kThreadBuild + t] : base.x);
        const float ang = sa == -2 ? (gi >= 0 ? grid.y : base.y) : (sa >= 0 ? fv[sa * kThreadBuild + t] : base.y);
        float dih = sx == -2 ? (gi >= 0 ? grid.z : base.z) : (sx >= 0 ? fv[sx * kThreadBuild + t] : base.z);
        if (sx >= 0)
            for (int q = S.cas_off[l]; q < S.cas_off[l + 1]; ++q) dih = dih + S.lig_shift[S.cas_atom[q]];
        float ca, sn_a, cd, sn_d;
        auto trig = [&](int c, int src, float deg, float* cs, float* sn) {
            if (trig_table(S, l, c, gi, src >= 0 ? gb[src * kThreadBuild + t] : -1, deg, cs, sn)) return;
            if (src >= 0) {
                const double b = (row[src] - S.gene_min[src]) / S.gene_del[src];
                const int exact = (b >= 0.0 && b < 2147483647.0) ? (int)rint(b) : -1;
                if (exact != gb[src * kThreadBuild + t] && trig_table(S, l, c, gi, exact, deg, cs, sn)) return;
            }
            trig_exact(deg, cs, sn);
        };
        trig(0, sa, ang, &ca, &sn_a);
        trig(1, sx, dih, &cd, &sn_d);
        float x[4], y[4], z[4], out[3];
        buildcc_refs(S, S.lig_rec[l], [&](int j, int k) { return pos[(3 * j + k) * kThreadBuild + t]; }, x, y, z);
        buildcc_place(x, y, z, dis, ca, sn_a, cd, sn_d, out);
        pos[(3 * l) * kThreadBuild + t] = out[0];
        pos[(3 * l + 1) * kThreadBuild + t] = out[1];
        pos[(3 * l + 2) * kThreadBuild + t] = out[2];
    }
    for (int k = 0; k < 3 * nl; ++k) xyz[(size_t)k * n + p] = pos[k * kThreadBuild + t];
}

// Partition function of the clustering step: sum of exp(-beta * app_evalue)
// (LIB/cluster.cpp:68-80), one partial per block.
__global__ void __launch_bounds__(kPassThreads)
cluster_z_kernel(int n, const double* __restrict__ e, double beta, double* __restrict__ part) {
    __shared__ double red[kPassThreads];
    double s = 0.0;
    for (int i = blockIdx.x * kPassThreads + threadIdx.x; i < n; i += gridDim.x * kPassThreads)
        s += exp(-1.0 * beta * e[i]);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = kPassThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__device__ __forceinline__ double sum_partials(const double* __restrict__ part, int nb) {
    double z = 0.0;
    for (int b = 0; b < nb; ++b) z += part[b];
    return z;
}

// Cluster c. Its head is next[c]: 0 for the first cluster, else the first chromosome the pass of
// cluster c - 1 left unclustered (n: none left, no cluster). Every later unclustered chromosome
// whose RMSD to the head is at most thr joins (member, rmsd); the others bid for next[c + 1].
// Each block leaves its members' count and their share of the cluster's ACF in part_cnt/part_acf
// at [c * gridDim.x + block].
__global__ void __launch_bounds__(kPassThreads)
cluster_pass_kernel(int n, int nl, int c, const float* __restrict__ xyz, float thr, float exit_sum,
                    const double* __restrict__ e, int temperature, double beta,
                    const double* __restrict__ part_z, int nb_z, int* __restrict__ member,
                    float* __restrict__ rmsd, int* __restrict__ next, double* __restrict__ part_acf,
                    int* __restrict__ part_cnt) {
    __shared__ float head_xyz[3 * kMaxLig];
    __shared__ double red[kPassThreads];
    __shared__ int red_n[kPassThreads / 32], red_next[kPassThreads / 32];
    __shared__ double z_sh;
    const int head = next[c];
    if (head >= n) return;
    const int m3 = 3 * nl;
    for (int k = threadIdx.x; k < m3; k += kPassThreads) head_xyz[k] = xyz[(size_t)k * n + head];
    if (threadIdx.x == 0) z_sh = temperature > 0 ? sum_partials(part_z, nb_z) : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        member[head] = head;
        rmsd[head] = 0.0f;
    }
    __syncthreads();
    const double z = z_sh, T = (double)temperature;
    const float nf = (float)nl;
    double acf = 0.0;
    int cnt = 0, first_left = n;
    for (int i = head + 1 + blockIdx.x * kPassThreads + threadIdx.x; i < n; i += gridDim.x * kPassThreads) {
        if (member[i] != -1) continue;
        // the sum of squared coordinate differences in the reference's order
        // (flexaids::sum_sq_distances_f's scalar form, LIB/simd_distance.h:712-713); partial sums
        // only grow, so a chromosome is given up once its partial sum is past exit_sum, a bound
        // above every sum whose RMSD is within thr
        float s = 0.0f;
        bool far = false;
        for (int a = 0; a < nl; ++a) {
            for (int k = 3 * a; k < 3 * a + 3; ++k) {
                const float d = xyz[(size_t)k * n + i] - head_xyz[k];
                s = s + d * d;
            }
            if (s > exit_sum) {
                far = true;
                break;
            }
        }
        const float r = far ? 0.0f : sqrtf(s / nf);
        if (!far && r <= thr) {
            member[i] = head;
            rmsd[i] = r;
            ++cnt;
            if (temperature > 0) {
                const double pi = exp(-1.0 * beta * e[i]) / z;
                acf += (pi * e[i]) + (T * pi * log(pi));
            } else {
                acf += e[i];
            }
        } else if (first_left == n) {
            first_left = i;   // this thread's chromosomes come in ascending order
        }
    }
    red[threadIdx.x] = acf;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        first_left = min(first_left, __shfl_xor_sync(0xffffffffu, first_left, o));
    }
    if (lane == 0) {
        red_n[w] = cnt;
        red_next[w] = first_left;
    }
    __syncthreads();
    for (int o = kPassThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        int tn = 0, tf = n;
        for (int k = 0; k < kPassThreads / 32; ++k) {
            tn += red_n[k];
            tf = min(tf, red_next[k]);
        }
        part_acf[(size_t)c * gridDim.x + blockIdx.x] = red[0];
        part_cnt[(size_t)c * gridDim.x + blockIdx.x] = tn;
        if (tf < n) atomicMin(&next[c + 1], tf);
    }
}

// Per cluster: head, frequency, TCF (the head's term) and ACF (the head's term plus its members'),
// LIB/cluster.cpp:116-170; and the RMSD between the heads of clusters a and b as calc_rmsd_chrom
// computes it for the .cad file (sum over atoms of sqrdist, LIB/geometry.cpp:96-102, then
// sqrt(sum / m), LIB/calc_rmsd_chrom.cpp:134-139).
__global__ void __launch_bounds__(kPassThreads)
cluster_finish_kernel(int n, int nl, int R, int nb, const float* __restrict__ xyz,
                      const double* __restrict__ e, int temperature, double beta,
                      const double* __restrict__ part_z, int nb_z, const int* __restrict__ next,
                      const double* __restrict__ part_acf, const int* __restrict__ part_cnt,
                      int* __restrict__ top, int* __restrict__ freq, double* __restrict__ tcf,
                      double* __restrict__ acf, float* __restrict__ head_rmsd, double* __restrict__ z_out) {
    __shared__ double z_sh;
    __shared__ int nc_sh;
    if (threadIdx.x == 0) {
        z_sh = temperature > 0 ? sum_partials(part_z, nb_z) : 0.0;
        int nc = 0;
        while (nc < R && next[nc] < n) ++nc;
        nc_sh = nc;
        *z_out = z_sh;
    }
    __syncthreads();
    const int nc = nc_sh;
    const double z = z_sh, T = (double)temperature;
    for (int c = threadIdx.x; c < R; c += kPassThreads) {
        if (c >= nc) {
            top[c] = 0;
            freq[c] = 0;
            tcf[c] = 0.0;
            acf[c] = 0.0;
            continue;
        }
        const int h = next[c];
        double lead;
        if (temperature > 0) {
            const double pj = exp(-1.0 * beta * e[h]) / z;
            lead = (double)((pj * e[h]) - (T * pj * log(pj)));
        } else {
            lead = e[h];
        }
        double s = lead;
        int f = 1;
        for (int b = 0; b < nb; ++b) {
            s += part_acf[(size_t)c * nb + b];
            f += part_cnt[(size_t)c * nb + b];
        }
        top[c] = h;
        freq[c] = f;
        tcf[c] = lead;
        acf[c] = s;
    }
    for (int q = threadIdx.x; q < nc * nc; q += kPassThreads) {
        const int a = q / nc, b = q % nc;
        const int ha = next[a], hb = next[b];
        float s = 0.0f;
        for (int l = 0; l < nl; ++l) {
            const float d0 = xyz[(size_t)(3 * l) * n + ha] - xyz[(size_t)(3 * l) * n + hb];
            const float d1 = xyz[(size_t)(3 * l + 1) * n + ha] - xyz[(size_t)(3 * l + 1) * n + hb];
            const float d2 = xyz[(size_t)(3 * l + 2) * n + ha] - xyz[(size_t)(3 * l + 2) * n + hb];
            s += d0 * d0 + d1 * d1 + d2 * d2;
        }
        head_rmsd[q] = (float)sqrt((double)(s / (float)nl));
    }
}

int cluster_blocks(int n) {
    const int want = (n + kPassThreads - 1) / kPassThreads;
    return want < 4 * 152 ? (want < 1 ? 1 : want) : 4 * 152;
}

cudaError_t launch_cluster(const DevSystem& S, const ClusterWork& C, cudaStream_t st) {
    const int n = C.n, nl = S.n_lig, nb = cluster_blocks(n);
    // at most 128 atoms and 100 genes (checked by the caller): 146 KB for 64 chromosomes
    const size_t tsmem = thread_build_smem(S);
    cudaError_t e = cudaFuncSetAttribute(cluster_build_thread_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tsmem);
    if (e != cudaSuccess) return e;
    cluster_build_thread_kernel<<<(n + kThreadBuild - 1) / kThreadBuild, kThreadBuild, tsmem, st>>>(S, n, C.ic,
                                                                                                  C.xyz, C.status);
    if (C.temperature > 0) cluster_z_kernel<<<nb, kPassThreads, 0, st>>>(n, C.e, C.beta, C.part_z);
    for (int c = 0; c < C.max_results; ++c)
        cluster_pass_kernel<<<nb, kPassThreads, 0, st>>>(n, nl, c, C.xyz, C.thr, C.exit_sum, C.e, C.temperature,
                                                         C.beta, C.part_z, nb, C.member, C.rmsd, C.next,
                                                         C.part_acf, C.part_cnt);
    cluster_finish_kernel<<<1, kPassThreads, 0, st>>>(n, nl, C.max_results, nb, C.xyz, C.e, C.temperature, C.beta,
                                                      C.part_z, nb, C.next, C.part_acf, C.part_cnt, C.top, C.freq,
                                                      C.tcf, C.acf, C.head_rmsd, C.z);
    return cudaGetLastError();
}

}  // namespace fxe
