// fxe_place.cuh — gene decode, IC assignment and buildcc of one pose by one warp: the part of
// the pose build that places the ligand. Included by the pose build (fxe_build.cu) and by the
// clustering kernels (fxe_cluster.cu), both compiled with --fmad=false so that the
// single-precision arithmetic is evaluated exactly as written, like the reference's buildcc
// (LIB/buildcc.cpp:6-134).
#pragma once

#include "fxe_common.cuh"

namespace fxe {

struct BuildShared {
    float ic[kMaxLig][3];
    float pos[kMaxLig][3];
    int cell[kMaxLig];          // per mobile atom
    float trig[kMaxLig][4];     // per ligand atom: cos, sin of its build angle, then of its dihedral
    float sc[kMaxSc][4];        // side-chain atoms: x, y, z, radius
    int rot[kMaxFlex];          // rotamer of each flexible residue
    double icv[64];
    int gbin[64];     // bin of each gene's value (its entry in the trigonometry tables)
    int gi;           // grid index of the pose
    int bad;
};

// cos and sin of the build angle x = (float)(deg * PI / 180) that buildcc forms from an IC in
// degrees (LIB/buildcc.cpp:80-100). The host tabulates, for the values the genes (or the grid, or
// the base ICs) give each atom, the degrees, x and the C library's cosf/sinf of x, so that
// coordinates match the reference built on the same host bit for bit. A table entry whose degrees
// equal deg gives the pair with no double-precision arithmetic at all; otherwise x is formed in
// double precision as buildcc forms it and the entry is used if its x equals x; else the
// correctly rounded values. gi is the pose's grid point, bin the bin of the gene that sets the
// angle (-1: none known); trig_table answers whether a table entry gave the pair.
__device__ __forceinline__ bool trig_table(const DevSystem& S, int l, int c, int gi, int bin, float deg, float* cs,
                                           float* sn) {
    const int k = 2 * l + c, src = S.trig_src[k];
    float4 e = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    bool have = false;
    if (src == -2) {
        if ((unsigned)gi < (unsigned)S.n_grid) {
            e = c == 0 ? S.grid_trig_a[gi] : S.grid_trig_d[gi];
            have = true;
        }
    } else {
        const int idx = src < 0 ? 0 : bin;
        if (idx >= 0 && idx < S.trig_cnt[k]) {
            e = S.trig_tab[S.trig_off[k] + idx];
            have = true;
        }
    }
    if (!have) return false;
    if (__float_as_int(e.w) == __float_as_int(deg) || __float_as_int(e.x) == __float_as_int((float)(deg * kPi / 180.0f))) {
        *cs = e.y;
        *sn = e.z;
        return true;
    }
    return false;
}

// Correctly rounded cos and sin of the build angle, for angles no table entry holds.
__device__ __forceinline__ void trig_exact(float deg, float* cs, float* sn) {
    const float x = (float)(deg * kPi / 180.0f);
    *cs = (float)cos((double)x);
    *sn = (float)sin((double)x);
}

__device__ __forceinline__ void trig_of(const DevSystem& S, int l, int c, int gi, int bin, float deg, float* cs,
                                        float* sn) {
    if (!trig_table(S, l, c, gi, bin, deg, cs, sn)) trig_exact(deg, cs, sn);
}

// The same for a warp's pose: its grid point and gene bins from the pose's shared state.
__device__ __forceinline__ void build_trig(const DevSystem& S, const BuildShared& sh, int l, int c, float deg,
                                           float* cs, float* sn) {
    const int src = S.trig_src[2 * l + c];
    trig_of(S, l, c, sh.gi, (src >= 0 && src < 64) ? sh.gbin[src] : -1, deg, cs, sn);
}

// genetoic's bin (LIB/gaboom.cpp:2887-2906) of gene value `gene` of gene g: the first running bin
// total at or above RandomDouble(gene), found by binary search in the totals the host precomputes.
__device__ __forceinline__ int gene_bin(const DevSystem& S, int g, int32_t gene) {
    const double u = gene / (2147483647.0 + 1.0);
    int lo = S.dec_off[g], hi = S.dec_off[g + 1];
    const int base = lo;
    while (lo < hi) {  // first entry >= u
        const int mid = (lo + hi) >> 1;
        if (S.dec_tab[mid] < u) lo = mid + 1; else hi = mid;
    }
    return lo - base;
}

// Step 1: genes -> ICs (genetoic, LIB/gaboom.cpp:2887-2906, as a binary search in the running bin
// totals the host precomputes) or ICs as given, then the clamp of eval_chromosome
// (LIB/gaboom.cpp:1845-1866) when `clamp`. The values go to sh.icv (genes < 64) and, when ic_out
// is set, to ic_out[g] (all genes); the warp's lanes share the genes.
__device__ __forceinline__ void decode_ics(const DevSystem& S, int p, const int32_t* __restrict__ genes,
                                           const double* __restrict__ ic_in, bool clamp,
                                           double* __restrict__ ic_out, BuildShared& sh, int lane) {
    const int ng = S.n_genes;
    for (int g = lane; g < ng; g += 32) {
        double v;
        if (genes) {
            const int bin = gene_bin(S, g, genes[(size_t)p * ng + g]);
            v = S.gene_min[g] + S.gene_del[g] * (double)bin;
            if (g < 64) sh.gbin[g] = bin;
        } else {
            v = ic_in[(size_t)p * ng + g];
            // the bin this value would come from; the table entry is used only if its angle matches
            const double b = (v - S.gene_min[g]) / S.gene_del[g];
            if (g < 64) sh.gbin[g] = (b >= 0.0 && b < 2147483647.0) ? (int)rint(b) : -1;
        }
        if (clamp) {
            if (v > S.gene_max[g]) v = S.gene_max[g];
            else if (v < S.gene_min[g]) v = S.gene_min[g];
        }
        if (ic_out) ic_out[g] = v;
        if (g < 64) sh.icv[g] = v;
    }
}

// Step 2, by lane 0 after decode_ics and a __syncwarp: the IC assignment of ic2cf
// (LIB/ic2cf.cpp:53-105: grid index, angle, dihedral with the rec[3] cascade, rotamer index).
// sh.ic must hold the ligand's base ICs; genes >= 64 are read from ic_row. Sets sh.gi, sh.rot and
// sh.bad (1: grid index out of range).
__device__ __forceinline__ void assign_ics(const DevSystem& S, BuildShared& sh, const double* ic_row) {
    const int ng = S.n_genes, nl = S.n_lig;
    for (int g = 0; g < ng; ++g) {
        const double v = g < 64 ? sh.icv[g] : ic_row[g];
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
}

// The reference points of buildcc (LIB/buildcc.cpp:20-60) for an atom with build references ref:
// the placed reference atoms (pos_of(j, k)) or, for a missing one, the frame points around
// FA->ori; each offset by 1e-10f.
template <typename PosOf>
__device__ __forceinline__ void buildcc_refs(const DevSystem& S, const int4& r, PosOf pos_of, float x[4], float y[4],
                                             float z[4]) {
    const float* ori = S.ori;
    const int ref[3] = {r.x, r.y, r.z};
    for (int i = 1; i <= 3; ++i) {
        const int j = ref[i - 1];
        if (j >= 0) {
            x[i] = pos_of(j, 0);
            y[i] = pos_of(j, 1);
            z[i] = pos_of(j, 2);
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
}

// buildcc's placement of one atom (LIB/buildcc.cpp:60-130) from its reference points, its
// distance and the cos/sin of its angle (ca, sa) and dihedral (cd, sd), single precision in the
// reference's order of operations.
__device__ __forceinline__ void buildcc_place(const float x[4], const float y[4], const float z[4], float dis,
                                              float ca, float sa, float cd, float sd, float out[3]) {
    float a = y[1] * (z[2] - z[3]) + y[2] * (z[3] - z[1]) + y[3] * (z[1] - z[2]);
    float b = z[1] * (x[2] - x[3]) + z[2] * (x[3] - x[1]) + z[3] * (x[1] - x[2]);
    float c = x[1] * (y[2] - y[3]) + x[2] * (y[3] - y[1]) + x[3] * (y[1] - y[2]);
    float op = sqrtf(a * a + b * b + c * c);
    float cx = a / op, cy = b / op, cz = c / op;
    a = x[2] - x[1];
    b = y[2] - y[1];
    c = z[2] - z[1];
    const float d = 1.0f / sqrtf(a * a + b * b + c * c);
    op = dis * d;
    const float xn = a * op, yn = b * op, zn = c * op;
    a = cx * cx;
    b = cy * cy;
    c = cz * cz;
    float ct = ca, st = -sa;
    op = 1.0f - ct;
    const float xk = (cx * cz * op - cy * st) * zn + ((1.0f - a) * ct + a) * xn + (cx * cy * op + cz * st) * yn;
    const float yk = (cy * cx * op - cz * st) * xn + ((1.0f - b) * ct + b) * yn + (cy * cz * op + cx * st) * zn;
    const float zk = (cz * cy * op - cx * st) * yn + ((1.0f - c) * ct + c) * zn + (cz * cx * op + cy * st) * xn;
    ct = cd;
    st = sd;
    op = 1.0f - ct;
    cx = (x[2] - x[1]) * d;
    cy = (y[2] - y[1]) * d;
    cz = (z[2] - z[1]) * d;
    a = cx * cx;
    b = cy * cy;
    c = cz * cz;
    out[0] = (cx * cz * op - cy * st) * zk + ((1.0f - a) * ct + a) * xk + (cx * cy * op + cz * st) * yk + x[1];
    out[1] = (cy * cx * op - cz * st) * xk + ((1.0f - b) * ct + b) * yk + (cy * cz * op + cx * st) * zk + y[1];
    out[2] = (cz * cy * op - cx * st) * yk + ((1.0f - c) * ct + c) * zk + (cz * cx * op + cy * st) * xk + z[1];
}

// buildcc (LIB/buildcc.cpp:6-134) of ligand atom l from its three build references (or the
// frame points around FA->ori), which must already be placed.
__device__ __forceinline__ void build_atom(const DevSystem& S, BuildShared& sh, int l) {
    float x[4], y[4], z[4], out[3];
    buildcc_refs(S, S.lig_rec[l], [&](int j, int k) { return sh.pos[j][k]; }, x, y, z);
    buildcc_place(x, y, z, sh.ic[l][0], sh.trig[l][0], sh.trig[l][1], sh.trig[l][2], sh.trig[l][3], out);
    sh.pos[l][0] = out[0];
    sh.pos[l][1] = out[1];
    sh.pos[l][2] = out[2];
}

// Step 3, by every lane after assign_ics and a __syncwarp: buildcc over the rebuild list. First
// the cos/sin pairs of every atom's angle and dihedral, which depend on its ICs only, one atom per
// lane; then the atoms of one dependency level are built by the warp's lanes at once (each atom's
// arithmetic is the same as in list order: its references are placed in earlier levels); without
// levels, lane 0 follows the list.
__device__ __forceinline__ void build_atoms(const DevSystem& S, BuildShared& sh, int lane) {
    for (int l = lane; l < S.n_lig; l += 32) {
        float c, s;
        build_trig(S, sh, l, 0, sh.ic[l][1], &c, &s);
        sh.trig[l][0] = c;
        sh.trig[l][1] = s;
        build_trig(S, sh, l, 1, sh.ic[l][2], &c, &s);
        sh.trig[l][2] = c;
        sh.trig[l][3] = s;
    }
    __syncwarp();
    if (S.n_levels > 0) {
        for (int v = 0; v < S.n_levels; ++v) {
            for (int i = S.level_off[v] + lane; i < S.level_off[v + 1]; i += 32) build_atom(S, sh, S.level_atom[i]);
            __syncwarp();
        }
    } else {
        if (lane == 0)
            for (int an = 0; an < S.n_build; ++an) build_atom(S, sh, S.build_order[an]);
        __syncwarp();
    }
}

// The ligand's base ICs into sh.ic and the per-pose state reset, before assign_ics.
__device__ __forceinline__ void reset_pose(const DevSystem& S, BuildShared& sh, int lane) {
    for (int l = lane; l < S.n_lig; l += 32) {
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
}

}  // namespace fxe
