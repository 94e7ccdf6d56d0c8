// fxe_prepare.cu — receptor preparation on the device, done once when a receptor enters the
// receptor cache (context creation):
//   * the cleft grid of generate_grid (LIB/generate_grid.cpp:18-107): the lattice points strictly
//     inside each cleft sphere, spheres in list order, a point dropped when an earlier sphere
//     produced a point with the same key (coordinates snapped to 0.001 A, GridKey,
//     LIB/maps.hpp:21-49);
//   * calc_cleftic (LIB/calc_cleftic.cpp:5-33): each grid point's distance, bond angle and
//     dihedral against the frame points ori + (1,0,0), ori, ori + (0,1,0), in single precision as
//     LIB/geometry.cpp computes them;
//   * index_protein's steady cell list of the rigid receptor atoms (LIB/Vcontacts.cpp:1584-1715):
//     each atom's 6.5 A cell, atoms grouped by cell in Calc order.
// Compiled with --fmad=false: every single-precision operation rounds as the reference's does.
//
// The lattice walks c[k] += spacer from min[k] (LIB/generate_grid.cpp:55-93); the value after m
// steps depends on m alone, so the host tabulates each axis by that same float addition and every
// thread reads its point's three axis values.
#include <cstdint>

#include "fxe_common.cuh"

namespace fxe {

long long scan_tmp_ints(long long n);
void scan_ints(const int* in, int* out, long long n, int* tmp, cudaStream_t st);

constexpr int kPrepThreads = 256;
constexpr unsigned long long kKeyEmpty = 0xFFFFFFFFFFFFFFFFull;

// GridKey's snap (std::round of v * 1000, halves away from zero), three 21-bit fields.
__device__ __forceinline__ unsigned long long grid_key(float x, float y, float z) {
    const long long ix = (long long)roundf(x * 1000.0f) + (1ll << 20);
    const long long iy = (long long)roundf(y * 1000.0f) + (1ll << 20);
    const long long iz = (long long)roundf(z * 1000.0f) + (1ll << 20);
    return ((unsigned long long)ix << 42) | ((unsigned long long)iy << 21) | (unsigned long long)iz;
}

__device__ __forceinline__ unsigned long long key_slot(unsigned long long k, unsigned long long mask) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    return k & mask;
}

__device__ bool key_present(const unsigned long long* set, unsigned long long mask, unsigned long long k) {
    unsigned long long i = key_slot(k, mask);
    for (unsigned long long n = 0; n <= mask; ++n, i = (i + 1) & mask) {
        const unsigned long long v = set[i];
        if (v == k) return true;
        if (v == kKeyEmpty) return false;
    }
    return false;
}

__device__ void key_insert(unsigned long long* set, unsigned long long mask, unsigned long long k) {
    unsigned long long i = key_slot(k, mask);
    for (unsigned long long n = 0; n <= mask; ++n, i = (i + 1) & mask) {
        const unsigned long long v = atomicCAS(set + i, kKeyEmpty, k);
        if (v == kKeyEmpty || v == k) return;
    }
}

// flag[t] = 1 for lattice point t (x fastest) strictly inside the sphere and, with check, not
// already produced by an earlier sphere.
__global__ void grid_mark_kernel(const float* __restrict__ ax, const float* __restrict__ ay, const float* __restrict__ az,
                                 int nx, int ny, int nz, float cx, float cy, float cz, float rr,
                                 const unsigned long long* __restrict__ set, unsigned long long mask, int check,
                                 int* __restrict__ flag) {
    const long long total = (long long)nx * ny * nz;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % nx);
        const long long r = t / nx;
        const int j = (int)(r % ny);
        const int k = (int)(r / ny);
        const float x = ax[i], y = ay[j], z = az[k];
        // sqrdist(center, c) (LIB/geometry.cpp:96-102)
        const float d0 = cx - x, d1 = cy - y, d2 = cz - z;
        const float d = d0 * d0 + d1 * d1 + d2 * d2;
        int f = d < rr;
        if (f && check) f = !key_present(set, mask, grid_key(x, y, z));
        flag[t] = f;
    }
}

// The flagged points, in lattice order, appended after `base` earlier points; their keys join the set.
__global__ void grid_emit_kernel(const float* __restrict__ ax, const float* __restrict__ ay, const float* __restrict__ az,
                                 int nx, int ny, int nz, const int* __restrict__ flag, const int* __restrict__ pos,
                                 long long base, float* __restrict__ xyz, unsigned long long* __restrict__ set,
                                 unsigned long long mask) {
    const long long total = (long long)nx * ny * nz;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        if (!flag[t]) continue;
        const int i = (int)(t % nx);
        const long long r = t / nx;
        const int j = (int)(r % ny);
        const int k = (int)(r / ny);
        const long long o = base + pos[t];
        xyz[3 * o] = ax[i];
        xyz[3 * o + 1] = ay[j];
        xyz[3 * o + 2] = az[k];
        key_insert(set, mask, grid_key(ax[i], ay[j], az[k]));
    }
}

// calc_cleftic of every grid point: distance (LIB/geometry.cpp:17-35), bndang (:115-131) and
// dihedral (:49-64) against ca = ori + (1,0,0), cb = ori, cc = ori + (0,1,0). The reference calls
// the C library's acosf and atan2f, which round correctly; here each is taken in double and
// rounded once to single precision.
__global__ void cleft_ic_kernel(const float* __restrict__ xyz, long long n, float ox, float oy, float oz,
                                float* __restrict__ ic) {
    const float ca[3] = {ox + 1.0f, oy, oz};
    const float cb[3] = {ox, oy, oz};
    const float cc[3] = {ox, oy + 1.0f, oz};
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const float ci[3] = {xyz[3 * p], xyz[3 * p + 1], xyz[3 * p + 2]};
        // distance(ci, ca)
        float delta = ci[0] - ca[0];
        float r2 = delta * delta;
        delta = ci[1] - ca[1];
        r2 += delta * delta;
        delta = ci[2] - ca[2];
        const float dis = sqrtf(r2 + delta * delta);
        // bndang(ci, ca, cb)
        float cosa = 0.0f, absu = 0.0f, absv = 0.0f;
        for (int i = 0; i < 3; ++i) {
            cosa += (ci[i] - ca[i]) * (cb[i] - ca[i]);
            absu += (ci[i] - ca[i]) * (ci[i] - ca[i]);
            absv += (cb[i] - ca[i]) * (cb[i] - ca[i]);
        }
        cosa /= sqrtf(absu * absv);
        const float acs = (float)acos((double)cosa);
        const float ang = (float)((double)acs * 180.0 / kPi);
        // dihedral(ci, ca, cb, cc)
        float r1[3], rb[3], r3[3], n1[3], n2[3];
        for (int i = 0; i < 3; ++i) {
            r1[i] = ca[i] - ci[i];
            rb[i] = cb[i] - ca[i];
            r3[i] = cc[i] - cb[i];
        }
        n1[0] = r1[1] * rb[2] - rb[1] * r1[2];
        n1[1] = -r1[0] * rb[2] + rb[0] * r1[2];
        n1[2] = r1[0] * rb[1] - rb[0] * r1[1];
        n2[0] = rb[1] * r3[2] - r3[1] * rb[2];
        n2[1] = -rb[0] * r3[2] + r3[0] * rb[2];
        n2[2] = rb[0] * r3[1] - r3[0] * rb[1];
        const float dn = n1[0] * r3[0] + n1[1] * r3[1] + n1[2] * r3[2];
        const float rr = rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2];
        const float psin = dn * sqrtf(rr);
        const float pcos = n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2];
        const float at = (float)atan2((double)psin, (double)pcos);
        ic[3 * p] = dis;
        ic[3 * p + 1] = ang;
        ic[3 * p + 2] = 57.2958f * at;
    }
}

static unsigned prep_grid(long long n) {
    long long b = (n + kPrepThreads - 1) / kPrepThreads;
    if (b > 16384) b = 16384;
    return (unsigned)(b > 0 ? b : 1);
}

// Device buffers of one grid generation: the largest sphere's lattice flags and scan, the key set.
size_t grid_scratch_bytes(long long max_lattice, long long key_slots) {
    const size_t a = (size_t)(max_lattice + 1) * sizeof(int) * 2;
    const size_t t = (size_t)scan_tmp_ints(max_lattice) * sizeof(int);
    return ((a + 255) & ~(size_t)255) + ((t + 255) & ~(size_t)255) + (size_t)key_slots * sizeof(unsigned long long);
}

// Sphere s's lattice: axis tables at axes + off[s] (x, then y, then z), dims[s]; centres and
// squared radii in spheres[4 s]; points go to xyz (device, capacity for every lattice point);
// n_points (device) gets the count. key_slots a power of two at least twice the points.
cudaError_t launch_cleft_grid(int n_spheres, const float* axes, const long long* off, const int* dims,
                              const float* spheres, long long max_lattice, long long key_slots, void* scratch,
                              float* xyz, long long* n_points_host, cudaStream_t st) {
    unsigned char* p = static_cast<unsigned char*>(scratch);
    const size_t a = (size_t)(max_lattice + 1) * sizeof(int) * 2;
    int* flag = reinterpret_cast<int*>(p);
    int* pos = flag + (max_lattice + 1);
    p += (a + 255) & ~(size_t)255;
    int* tmp = reinterpret_cast<int*>(p);
    p += ((size_t)scan_tmp_ints(max_lattice) * sizeof(int) + 255) & ~(size_t)255;
    auto* set = reinterpret_cast<unsigned long long*>(p);
    const unsigned long long mask = (unsigned long long)key_slots - 1;
    cudaError_t e = cudaMemsetAsync(set, 0xFF, (size_t)key_slots * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    long long base = 0;
    for (int s = 0; s < n_spheres; ++s) {
        const int nx = dims[3 * s], ny = dims[3 * s + 1], nz = dims[3 * s + 2];
        const long long total = (long long)nx * ny * nz;
        if (total <= 0) continue;
        const float* ax = axes + off[s];
        const float* ay = ax + nx;
        const float* az = ay + ny;
        grid_mark_kernel<<<prep_grid(total), kPrepThreads, 0, st>>>(ax, ay, az, nx, ny, nz, spheres[4 * s], spheres[4 * s + 1],
                                                                     spheres[4 * s + 2], spheres[4 * s + 3], set, mask, s > 0,
                                                                     flag);
        scan_ints(flag, pos, total, tmp, st);
        grid_emit_kernel<<<prep_grid(total), kPrepThreads, 0, st>>>(ax, ay, az, nx, ny, nz, flag, pos, base, xyz, set, mask);
        int added = 0;
        if ((e = cudaMemcpyAsync(&added, pos + total, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
        base += added;
    }
    *n_points_host = base;
    return cudaGetLastError();
}

void launch_cleft_ic(const float* xyz, long long n, const float ori[3], float* ic, cudaStream_t st) {
    if (n > 0) cleft_ic_kernel<<<prep_grid(n), kPrepThreads, 0, st>>>(xyz, n, ori[0], ori[1], ori[2], ic);
}

// --- steady cell list ------------------------------------------------------------------------

// cell[i] of each rigid receptor atom ((int)((x - gmin) / 6.5) per axis, LIB/Vcontacts.cpp:1648-1655),
// -1 for side-chain atoms; counts per cell; bad[0] set when an atom falls outside the grid.
__global__ void cell_index_kernel(const float4* __restrict__ pos, const int* __restrict__ rec_mob, int n, float g0, float g1,
                                  float g2, int dim, int* __restrict__ cell, int* __restrict__ count, int* __restrict__ bad) {
    const long long dim2 = (long long)dim * dim, dim3 = dim2 * dim;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (rec_mob && rec_mob[i] >= 0) {
            cell[i] = -1;
            continue;
        }
        const float4 q = pos[i];
        const long long bi = (long long)(int)((q.x - g0) / kCell) * dim2 + (long long)(int)((q.y - g1) / kCell) * dim +
                             (int)((q.z - g2) / kCell);
        if (bi < 0 || bi >= dim3) {
            atomicExch(bad, 1);
            cell[i] = -1;
            continue;
        }
        cell[i] = (int)bi;
        atomicAdd(count + bi, 1);
    }
}

// Atoms grouped by cell in Calc order: one warp per cell walks the atoms in order, 32 at a time,
// and places the cell's members at its offset (ballot ranks keep the order).
__global__ void cell_fill_kernel(const float4* __restrict__ pos, const int* __restrict__ cell, int n,
                                 const int* __restrict__ start, long long n_cells, const int* __restrict__ cell_of_rank,
                                 int n_busy, int* __restrict__ catom, float4* __restrict__ cpos) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int w = blockIdx.x * wpb + (threadIdx.x >> 5); w < n_busy; w += gridDim.x * wpb) {
        const int c = cell_of_rank[w];
        int o = start[c];
        for (int i0 = 0; i0 < n; i0 += 32) {
            const int i = i0 + lane;
            const bool mine = i < n && cell[i] == c;
            const unsigned m = __ballot_sync(0xffffffffu, mine);
            if (mine) {
                const int d = o + __popc(m & lanemask_lt());
                catom[d] = i;
                cpos[d] = pos[i];
            }
            o += __popc(m);
        }
    }
    (void)n_cells;
}

// busy[c] = 1 for cells with atoms (scanned into the list of busy cells).
__global__ void cell_busy_kernel(const int* __restrict__ count, long long n_cells, int* __restrict__ busy) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n_cells; c += (long long)gridDim.x * blockDim.x)
        busy[c] = count[c] > 0;
}

__global__ void cell_busy_list_kernel(const int* __restrict__ busy, const int* __restrict__ bpos, long long n_cells,
                                      int* __restrict__ list) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n_cells; c += (long long)gridDim.x * blockDim.x)
        if (busy[c]) list[bpos[c]] = (int)c;
}

size_t cell_scratch_bytes(int n, long long n_cells) {
    const long long big = n_cells + 1 > n ? n_cells + 1 : n;
    return (size_t)(n + 3 * (n_cells + 1) + 8) * sizeof(int) + (size_t)scan_tmp_ints(big) * sizeof(int) + 1024;
}

// The steady cell list of the rigid atoms: start[n_cells + 1] (CSR offsets), catom / cpos (the
// rigid atoms grouped by cell, Calc order inside a cell). Waits for the result; *bad_host is set
// when an atom lies outside the grid.
cudaError_t launch_cell_list(const float4* pos, const int* rec_mob, int n, const float gmin[3], int dim, void* scratch,
                             int* start, int* catom, float4* cpos, int* bad_host, cudaStream_t st) {
    const long long n_cells = (long long)dim * dim * dim;
    int* cell = static_cast<int*>(scratch);
    int* count = cell + n;
    int* busy = count + (n_cells + 1);
    int* bpos = busy + (n_cells + 1);
    int* bad = bpos + (n_cells + 1);
    int* tmp = bad + 8;
    cudaError_t e = cudaMemsetAsync(count, 0, (size_t)(n_cells + 1) * sizeof(int), st);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(bad, 0, sizeof(int), st)) != cudaSuccess) return e;
    cell_index_kernel<<<prep_grid(n), kPrepThreads, 0, st>>>(pos, rec_mob, n, gmin[0], gmin[1], gmin[2], dim, cell, count, bad);
    scan_ints(count, start, n_cells, tmp, st);
    cell_busy_kernel<<<prep_grid(n_cells), kPrepThreads, 0, st>>>(count, n_cells, busy);
    scan_ints(busy, bpos, n_cells, tmp, st);
    cell_busy_list_kernel<<<prep_grid(n_cells), kPrepThreads, 0, st>>>(busy, bpos, n_cells, count);
    int n_busy = 0;
    if ((e = cudaMemcpyAsync(&n_busy, bpos + n_cells, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(bad_host, bad, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    if (*bad_host || n_busy <= 0) return cudaSuccess;
    // `count` now lists the busy cells
    cell_fill_kernel<<<prep_grid((long long)n_busy * 32), kPrepThreads, 0, st>>>(pos, cell, n, start, n_cells, count, n_busy,
                                                                                catom, cpos);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

}  // namespace fxe
