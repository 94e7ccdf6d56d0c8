// fxe_ensemble.cu — the GA ensemble the reference hands to statmech, assembled on the device:
// every generation's population (the snapshots, LIB/gaboom.cpp:494), sorted by energy
// (QuickSort, :520; ties here keep snapshot order), then remove_dups (:2728-2747): a chromosome is
// dropped when every decoded gene lies within 0.1 of the last chromosome kept.
//
// Sort: least-significant-digit radix sort of the energies' order-preserving 64-bit images, 4 bits
// a pass (16 passes), each pass a per-block digit count, one scan of the counts and a stable
// scatter (a block's elements ranked by warp match and per-warp counts), so equal energies keep
// their input order.
//
// remove_dups is a chain: whether chromosome i is kept depends on which one was kept last. Runs of
// identical chromosomes (a survivor sits in the population for many generations) are collapsed
// first: a chromosome identical to its predecessor is always dropped and never becomes the last one
// kept. Over the remaining run heads, next(t) = the first later head that is not within 0.1 of head
// t (a bounded scan per thread, then one warp per unresolved head scanning 32 at a time); the kept
// heads are the path 0, next(0), next(next(0)), ..., marked by pointer jumping in log2(M) rounds.
#include <cstdint>

#include "fxe_place.cuh"

namespace fxe {

constexpr int kEnsThreads = 256;
constexpr int kScanThreads = 1024;
constexpr int kNearScan = 32;          // heads a thread tests before handing its head to a warp
constexpr double kDupTol = 0.1;        // LIB/gaboom.cpp:2737

// Order-preserving image of a double (NaN placed after +infinity, -0 with +0).
__device__ __forceinline__ unsigned long long order_key(double e) {
    if (e != e) return 0xFFFFFFFFFFFFFFFFull;
    if (e == 0.0) return 0x8000000000000000ull;   // -0 and +0 compare equal
    const unsigned long long b = (unsigned long long)__double_as_longlong(e);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void ens_keys_kernel(const double* __restrict__ e, long long n, unsigned long long* __restrict__ key,
                                int* __restrict__ val) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        key[i] = order_key(e[i]);
        val[i] = (int)i;
    }
}

// --- exclusive scan of int counts (n entries, total written to out[n]) -------------------------

__device__ __forceinline__ int block_excl_scan(int v, int* wsum, int* total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = lane < nw ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) wsum[lane] = s;
    }
    __syncthreads();
    const int before = w > 0 ? wsum[w - 1] : 0;
    *total = wsum[nw - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) scan_block_kernel(const int* __restrict__ in, int* __restrict__ out, long long n,
                                                                  int* __restrict__ bsum) {
    __shared__ int wsum[32];
    const long long i = blockIdx.x * (long long)kScanThreads + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    int tot;
    const int ex = block_excl_scan(v, wsum, &tot);
    if (i < n) out[i] = ex;
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// One block: exclusive scan of the nb block sums in place, the grand total to *total.
__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(int* __restrict__ bsum, int nb, int* __restrict__ total) {
    __shared__ int wsum[32];
    const int per = (nb + kScanThreads - 1) / kScanThreads;
    const int b0 = threadIdx.x * per;
    int s = 0;
    for (int k = 0; k < per && b0 + k < nb; ++k) s += bsum[b0 + k];
    int tot;
    int run = block_excl_scan(s, wsum, &tot);
    for (int k = 0; k < per && b0 + k < nb; ++k) {
        const int v = bsum[b0 + k];
        bsum[b0 + k] = run;
        run += v;
    }
    if (threadIdx.x == 0) *total = tot;
}

__global__ void scan_add_kernel(int* __restrict__ out, long long n, const int* __restrict__ bsum) {
    const long long i = blockIdx.x * (long long)kScanThreads + threadIdx.x;
    if (i < n) out[i] += bsum[blockIdx.x];
}

// tmp: at least scan_tmp_ints(n) ints. out: n + 1 ints (out[n] = the total).
static long long scan_blocks(long long n) { return (n + kScanThreads - 1) / kScanThreads; }
long long scan_tmp_ints(long long n) { return scan_blocks(n > 0 ? n : 1) + 1; }

void scan_ints(const int* in, int* out, long long n, int* tmp, cudaStream_t st) {
    const long long nb = scan_blocks(n > 0 ? n : 1);
    scan_block_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(in, out, n, tmp);
    scan_sums_kernel<<<1, kScanThreads, 0, st>>>(tmp, (int)nb, out + n);
    scan_add_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(out, n, tmp);
}

// --- radix sort passes --------------------------------------------------------------------------

__global__ void __launch_bounds__(kEnsThreads) radix_hist_kernel(const unsigned long long* __restrict__ key, long long n, int shift,
                                                                 int* __restrict__ hist) {
    __shared__ int cnt[16];
    if (threadIdx.x < 16) cnt[threadIdx.x] = 0;
    __syncthreads();
    const long long i = blockIdx.x * (long long)kEnsThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(int)((key[i] >> shift) & 15ull)], 1);
    __syncthreads();
    if (threadIdx.x < 16) hist[(long long)threadIdx.x * gridDim.x + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(kEnsThreads) radix_scatter_kernel(const unsigned long long* __restrict__ kin, const int* __restrict__ vin,
                                                                    unsigned long long* __restrict__ kout, int* __restrict__ vout,
                                                                    long long n, int shift, const int* __restrict__ offs) {
    __shared__ int wcnt[kEnsThreads / 32][16];
    const long long i = blockIdx.x * (long long)kEnsThreads + threadIdx.x;
    const int w = threadIdx.x >> 5;
    const bool ok = i < n;
    const unsigned long long k = ok ? kin[i] : 0ull;
    const int dg = ok ? (int)((k >> shift) & 15ull) : 16;
    const unsigned peers = __match_any_sync(0xffffffffu, dg);
    const int rank = __popc(peers & lanemask_lt());
    if (threadIdx.x < (kEnsThreads / 32) * 16) wcnt[threadIdx.x >> 4][threadIdx.x & 15] = 0;
    __syncthreads();
    if (ok && rank == 0) wcnt[w][dg] = __popc(peers);
    __syncthreads();
    if (ok) {
        int before = 0;
        for (int u = 0; u < w; ++u) before += wcnt[u][dg];
        const long long dst = (long long)offs[(long long)dg * gridDim.x + blockIdx.x] + before + rank;
        kout[dst] = k;
        vout[dst] = vin[i];
    }
}

// --- the chain over run heads -------------------------------------------------------------------

__device__ __forceinline__ bool within_tol(const double* __restrict__ a, const double* __restrict__ b, int ng) {
    for (int q = 0; q < ng; ++q)
        if (!(fabs(a[q] - b[q]) < kDupTol)) return false;
    return true;
}

// head[p] = 1 where sorted chromosome p differs from p - 1 in some decoded gene.
__global__ void ens_heads_kernel(const double* __restrict__ ic, long long n, int ng, int* __restrict__ head) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        int h = 1;
        if (p > 0) {
            h = 0;
            const double* a = ic + p * ng;
            const double* b = a - ng;
            for (int q = 0; q < ng; ++q)
                if (a[q] != b[q]) { h = 1; break; }
        }
        head[p] = h;
    }
}

// H[t]: the sorted position of head t.
__global__ void ens_compact_kernel(const int* __restrict__ flag, const int* __restrict__ pos, long long n, int* __restrict__ out) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
        if (flag[p]) out[pos[p]] = (int)p;
}

__global__ void ens_next_kernel(const double* __restrict__ ic, int ng, const int* __restrict__ H, const int* __restrict__ Mp,
                                int* __restrict__ nxt, int* __restrict__ far_list, int* __restrict__ far_n) {
    const int M = *Mp;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        const double* a = ic + (long long)H[t] * ng;
        int r = -1;
        const int last = t + kNearScan < M - 1 ? t + kNearScan : M - 1;
        for (int s = t + 1; s <= last; ++s)
            if (!within_tol(ic + (long long)H[s] * ng, a, ng)) { r = s; break; }
        if (r < 0) {
            if (last >= M - 1) r = M;
            else far_list[atomicAdd(far_n, 1)] = t;
        }
        nxt[t] = r;
    }
}

// One warp per head whose next head lies beyond the bounded scan: 32 later heads at a time.
__global__ void ens_next_far_kernel(const double* __restrict__ ic, int ng, const int* __restrict__ H, const int* __restrict__ Mp,
                                    int* __restrict__ nxt, const int* __restrict__ far_list, const int* __restrict__ far_n) {
    const int M = *Mp, nf = *far_n;
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int u = blockIdx.x * wpb + (threadIdx.x >> 5); u < nf; u += gridDim.x * wpb) {
        const int t = far_list[u];
        const double* a = ic + (long long)H[t] * ng;
        int r = M;
        for (int base = t + kNearScan + 1; base < M; base += 32) {
            const int s = base + lane;
            const bool hit = s < M && !within_tol(ic + (long long)H[s] * ng, a, ng);
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (m) {
                r = base + __ffs(m) - 1;
                break;
            }
        }
        if (lane == 0) nxt[t] = r;
    }
}

__global__ void ens_path_init_kernel(const int* __restrict__ nxt, const int* __restrict__ Mp, int* __restrict__ jump,
                                     uint8_t* __restrict__ on) {
    const int M = *Mp;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        jump[t] = nxt[t];
        on[t] = t == 0;
    }
}

// One pointer-jumping round: every marked head marks the head 2^r steps along the chain.
__global__ void ens_path_round_kernel(const int* __restrict__ jin, int* __restrict__ jout, const uint8_t* __restrict__ oin,
                                      uint8_t* __restrict__ oout, const int* __restrict__ Mp) {
    const int M = *Mp;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        const int j = jin[t];
        if (oin[t]) {
            oout[t] = 1;
            if (j < M) oout[j] = 1;
        }
        jout[t] = j < M ? jin[j] : M;
    }
}

// kept[t] = 1 for the kept heads (as ints, for the scan), 0 past M.
__global__ void ens_kept_flags_kernel(const uint8_t* __restrict__ on, const int* __restrict__ Mp, long long n, int* __restrict__ flag) {
    const int M = *Mp;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        flag[t] = t < M ? (int)on[t] : 0;
}

// Sorted ICs from ICs given in input order.
__global__ void ens_gather_ic_kernel(const double* __restrict__ ic_in, const int* __restrict__ order, long long n, int ng,
                                     double* __restrict__ ic_out) {
    const long long total = n * ng;
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total; x += (long long)gridDim.x * blockDim.x) {
        const long long p = x / ng;
        const int q = (int)(x - p * ng);
        ic_out[x] = ic_in[(long long)order[p] * ng + q];
    }
}

// Sorted ICs decoded from int32 genes in input order, clamped as eval_chromosome leaves them.
__global__ void ens_decode_kernel(DevSystem S, const int32_t* __restrict__ genes, const int* __restrict__ order, long long n,
                                  double* __restrict__ ic_out) {
    const int ng = S.n_genes;
    const long long total = n * ng;
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total; x += (long long)gridDim.x * blockDim.x) {
        const long long p = x / ng;
        const int q = (int)(x - p * ng);
        double v = S.gene_min[q] + S.gene_del[q] * (double)gene_bin(S, q, genes[(long long)order[p] * ng + q]);
        if (v > S.gene_max[q]) v = S.gene_max[q];
        else if (v < S.gene_min[q]) v = S.gene_min[q];
        ic_out[x] = v;
    }
}

// The kept chromosomes: their sorted positions (kept_pos) -> input indices, energies and ICs.
__global__ void ens_emit_kernel(const int* __restrict__ H, const int* __restrict__ flag, const int* __restrict__ pos,
                                const int* __restrict__ Mp, const int* __restrict__ order, const double* __restrict__ e_in,
                                const double* __restrict__ ic_sorted, int ng, long long* __restrict__ idx_out,
                                double* __restrict__ e_out, double* __restrict__ ic_out) {
    const int M = *Mp;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        if (!flag[t]) continue;
        const int k = pos[t];
        const int p = H[t];
        const int src = order[p];
        if (idx_out) idx_out[k] = src;
        if (e_out) e_out[k] = e_in[src];
        if (ic_out)
            for (int q = 0; q < ng; ++q) ic_out[(long long)k * ng + q] = ic_sorted[(long long)p * ng + q];
    }
}

// --- driver ---------------------------------------------------------------------------------

static unsigned grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b > 16384) b = 16384;
    return (unsigned)(b > 0 ? b : 1);
}

// The scratch buffers of one assembly, carved from one allocation in a fixed order; with base
// null only the size is counted (ensemble_scratch_bytes), so sizing and carving cannot disagree.
struct EnsScratch {
    unsigned long long *k0, *k1;
    int *v0, *v1, *hist, *stmp, *head;
    double* ics;
    uint8_t* oa;
    int* cnt;
    size_t bytes = 0;

    template <typename T>
    T* take(unsigned char* base, size_t count) {
        T* q = base ? reinterpret_cast<T*>(base + bytes) : nullptr;
        bytes += (count * sizeof(T) + 255) & ~(size_t)255;
        return q;
    }
    void carve(unsigned char* base, long long n, int ng) {
        const long long nb = (n + kEnsThreads - 1) / kEnsThreads;
        const long long st_n = 16 * nb > n + 1 ? 16 * nb : n + 1;
        bytes = 0;
        k0 = take<unsigned long long>(base, n);
        k1 = take<unsigned long long>(base, n);
        v0 = take<int>(base, n);
        v1 = take<int>(base, n);
        hist = take<int>(base, 32 * nb + 1);          // digit counts [16 nb], their scan [16 nb + 1]
        stmp = take<int>(base, scan_tmp_ints(st_n));
        ics = take<double>(base, (size_t)n * ng);
        head = take<int>(base, 6 * (n + 1));           // head flags, positions, H, next, two jump arrays
        oa = take<uint8_t>(base, 2 * (size_t)n);       // two mark arrays
        cnt = take<int>(base, 4);                      // M, far count
    }
};

size_t ensemble_scratch_bytes(long long n, int ng) {
    EnsScratch s;
    s.carve(nullptr, n > 0 ? n : 1, ng);
    return s.bytes;
}

// Sorts n energies, collapses identical runs, runs the chain and writes the kept chromosomes
// (input indices, energies, ICs; each may be null) in energy order; *d_kept (device) gets their
// count. ICs come from ic_in (n * ng, input order) or, when null, from genes decoded with S.
// scratch: ensemble_scratch_bytes(n, ng) bytes.
cudaError_t launch_ensemble(long long n, int ng, const double* e_in, const double* ic_in, const DevSystem* S,
                            const int32_t* genes, void* scratch, long long* idx_out, double* e_out, double* ic_out,
                            int* d_kept, cudaStream_t st) {
    if (n <= 0) return cudaMemsetAsync(d_kept, 0, sizeof(int), st);
    const long long nb = (n + kEnsThreads - 1) / kEnsThreads;
    EnsScratch sc;
    sc.carve(static_cast<unsigned char*>(scratch), n, ng);
    unsigned long long *k0 = sc.k0, *k1 = sc.k1;
    int *v0 = sc.v0, *v1 = sc.v1;
    int* hist = sc.hist;
    int* hoff = hist + 16 * nb;
    int* stmp = sc.stmp;
    double* ics = sc.ics;
    int* head = sc.head;
    int* hpos = head + (n + 1);
    int* H = hpos + (n + 1);
    int* nxt = H + (n + 1);
    int* ja = nxt + (n + 1);
    int* jb = ja + (n + 1);
    uint8_t* oa = sc.oa;
    uint8_t* ob = oa + n;
    int* cnt = sc.cnt;                                       // [0] M, [1] far count
    int* kept_flag = head;                                   // reused once the heads are compacted
    int* kept_pos = hpos;

    ens_keys_kernel<<<grid_for(n, kEnsThreads), kEnsThreads, 0, st>>>(e_in, n, k0, v0);
    for (int pass = 0; pass < 16; ++pass) {
        const int shift = 4 * pass;
        radix_hist_kernel<<<(unsigned)nb, kEnsThreads, 0, st>>>(k0, n, shift, hist);
        scan_ints(hist, hoff, 16 * nb, stmp, st);
        radix_scatter_kernel<<<(unsigned)nb, kEnsThreads, 0, st>>>(k0, v0, k1, v1, n, shift, hoff);
        unsigned long long* tk = k0; k0 = k1; k1 = tk;
        int* tv = v0; v0 = v1; v1 = tv;
    }
    // v0: input index at each sorted position
    if (ic_in) ens_gather_ic_kernel<<<grid_for(n * ng, kEnsThreads), kEnsThreads, 0, st>>>(ic_in, v0, n, ng, ics);
    else ens_decode_kernel<<<grid_for(n * ng, kEnsThreads), kEnsThreads, 0, st>>>(*S, genes, v0, n, ics);
    ens_heads_kernel<<<grid_for(n, kEnsThreads), kEnsThreads, 0, st>>>(ics, n, ng, head);
    scan_ints(head, hpos, n, stmp, st);
    ens_compact_kernel<<<grid_for(n, kEnsThreads), kEnsThreads, 0, st>>>(head, hpos, n, H);
    cudaError_t e = cudaMemcpyAsync(cnt, hpos + n, sizeof(int), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(cnt + 1, 0, sizeof(int), st)) != cudaSuccess) return e;
    // heads: at most n; the kernels read M from the device
    ens_next_kernel<<<grid_for(n, kEnsThreads), kEnsThreads, 0, st>>>(ics, ng, H, cnt, nxt, ja, cnt + 1);
    ens_next_far_kernel<<<grid_for(n * 32, kEnsThreads), kEnsThreads, 0, st>>>(ics, ng, H, cnt, nxt, ja, cnt + 1);
    ens_path_init_kernel<<<grid_for(n, kEnsThreads), kEnsThreads, 0, st>>>(nxt, cnt, ja, oa);
    int rounds = 0;
    while ((1ll << rounds) < n) ++rounds;
    for (int r = 0; r < rounds; ++r) {
        if ((e = cudaMemsetAsync(ob, 0, (size_t)n, st)) != cudaSuccess) return e;
        ens_path_round_kernel<<<grid_for(n, kEnsThreads), kEnsThreads, 0, st>>>(ja, jb, oa, ob, cnt);
        int* tj = ja; ja = jb; jb = tj;
        uint8_t* to = oa; oa = ob; ob = to;
    }
    ens_kept_flags_kernel<<<grid_for(n, kEnsThreads), kEnsThreads, 0, st>>>(oa, cnt, n, kept_flag);
    scan_ints(kept_flag, kept_pos, n, stmp, st);
    ens_emit_kernel<<<grid_for(n, kEnsThreads), kEnsThreads, 0, st>>>(H, kept_flag, kept_pos, cnt, v0, e_in, ics, ng, idx_out,
                                                                      e_out, ic_out);
    if ((e = cudaMemcpyAsync(d_kept, kept_pos + n, sizeof(int), cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace fxe
