// fxe_ga.cu — the GA generation on the device: breeding (roulette selection, crossover,
// mutation on the int32 genes) and replacement, one block per job, for populations kept in HBM.
//
// Semantics follow the reference's operators:
//   * fitness of the population sorted by energy (calculate_fitness, LIB/gaboom.cpp:1627-1760):
//     LINEAR P - i; PSHARE (the reference's default) (P - i) / niche count, the niche count
//     summing 1 - (rmsp / sig_share)^alpha over the chromosomes within sig_share; SMFREE the
//     blend of rank and Boltzmann weight over the same niche count. Under PSHARE the population
//     is walked in fitness order after a generation (LIB/gaboom.cpp:498-499);
//   * roulette_wheel: r = u * sum(fitness), the first index whose running fitness sum exceeds r
//     (LIB/gaboom.cpp:1158-1186);
//   * the reproduce loop (LIB/gaboom.cpp:909-1000): pairs of parents, adaptive probabilities
//     (adapt_prob, :848-880) when asked, crossover with probability crossprob, both children
//     mutated, until nnew children exist;
//   * crossover: the reference's two-point bit crossover over the genes' 32-bit strings, with
//     its choice of genes and bit points, inside genes or at gene boundaries
//     (LIB/gaboom.cpp:2517-2614);
//   * mutate: every bit of every gene flipped with probability mutprob (LIB/gaboom.cpp:2620-2641);
//   * replacement (LIB/gaboom.cpp:1023-1033): BOOM merges parents and children and keeps the best
//     P; STEADY puts the children in place of the worst parents.
// The reference draws from a random_device-seeded generator, so its trajectories cannot be
// replayed; here every draw is a counter-based hash of (job seed, generation, child, draw), so a
// job's trajectory depends on its seed alone — the same whether it runs alone or among others.
// Duplicate rejection (LIB/gaboom.cpp:977-1018 and the populate loop, :1936-1978): children and
// initial chromosomes whose hash_genes signature the job has seen are dropped, as by the
// reference's default (duplicates = false).
#include <cstdint>

#include "fxe_common.cuh"

namespace fxe {

// SplitMix64 finaliser (Steele, Lea and Flood, OOPSLA 2014) of a 64-bit counter.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// The 53 random bits of draw `k` of stream `s` of a job.
__device__ __forceinline__ uint64_t uniform_bits(uint64_t seed, uint64_t s, uint64_t k) {
    return mix64(seed ^ mix64(s * 0x100000001B3ull + k)) >> 11;
}

// Uniform double in [0, 1) for draw `k` of stream `s` of a job: its 53 bits times 2^-53 (both
// steps exact).
__device__ __forceinline__ double uniform(uint64_t seed, uint64_t s, uint64_t k) {
    return (double)uniform_bits(seed, s, k) * 0x1.0p-53;
}

// A probability p with the integer form of the test u < p for draws u = b 2^-53 (b < 2^53 an
// integer): u < p exactly when b < ceil(p 2^53), the scaling by 2^53 being exact. Tests with it
// stay on the integer units (a mutation makes 32 such tests per gene).
struct DrawThreshold {
    double p;
    uint64_t bits;
};
__device__ __forceinline__ DrawThreshold draw_threshold(double p) {
    const double t = p * 0x1.0p53;
    uint64_t b = 0;                                  // p <= 0 or NaN: no draw is below
    if (t >= 0x1.0p53) b = 1ull << 53;               // p >= 1: every draw is
    else if (t > 0.0) b = (uint64_t)ceil(t);
    return {p, b};
}

constexpr int kGaThreads = 256;
// The one-block-per-job sorts (replacement, fitness): a wider block, so that each bitonic stage
// is a couple of exchanges per thread.
constexpr int kGaSortThreads = 1024;
constexpr int kGaMaxSort = 4096;   // 2P entries sorted in shared memory: P <= 2048

// Order-preserving 64-bit image of a double that is not a NaN: the images compare as unsigned
// integers in the order the values compare (-0 and +0, which compare equal, share one image), so
// the sorts below run on the integer units rather than on the narrow double-precision pipe.
__device__ __forceinline__ uint64_t order_key(double x) {
    uint64_t b = (uint64_t)__double_as_longlong(x);
    if ((b << 1) == 0) b = 0;
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Ascending bitonic sort of (key, index) pairs in shared memory, n a power of two.
__device__ void bitonic_sort(uint64_t* key, int* idx, int n) {
    for (int k = 2; k <= n; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    const uint64_t a = key[i], b = key[l];
                    const int ia = idx[i], ib = idx[l];
                    // order by key, then by index, so equal energies keep a fixed order
                    const bool gt = a > b || (a == b && ia > ib);
                    if (gt == up) {
                        key[i] = b; key[l] = a;
                        idx[i] = ib; idx[l] = ia;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// roulette_wheel (LIB/gaboom.cpp:1158-1186) over the fitness in roulette order: the first
// position whose running sum exceeds r = u * total, the last position if none does, and a
// uniform position when the total is not positive.
__device__ __forceinline__ int roulette(const GaJob& J, double u) {
    const int P = J.P;
    const double tot = J.fstat[0];
    if (!(tot > 0.0)) return (int)(u * (double)P) % P;
    const double r = u * tot;
    int lo = 0, hi = P - 1;   // smallest k with fcum[k] > r
    if (!(J.fcum[P - 1] > r)) return P - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (J.fcum[mid] > r) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// genetoic (LIB/gaboom.cpp:2887-2906): the first running bin total at or above u.
__device__ __forceinline__ double gene_ic(const GaJob& J, int g, int32_t gene) {
    const double u = gene / (2147483647.0 + 1.0);
    // the totals are positive: as signed 64-bit integers their bit patterns compare with u's as
    // the values do (a negative gene's u lies below them all), on the integer units
    const long long ub = __double_as_longlong(u);
    int lo = J.dec_off[g], hi = J.dec_off[g + 1];
    const int base = lo;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__double_as_longlong(J.dec_tab[mid]) < ub) lo = mid + 1;
        else hi = mid;
    }
    return J.gene_min[g] + J.gene_del[g] * (double)(lo - base);
}

// hash_genes (LIB/gaboom.cpp:1040-1045) with the C++ library's identity hash of int32.
__device__ __forceinline__ uint64_t signature(const GaJob& J, const int32_t* genes) {
    uint64_t h = 0;
    for (int i = 0; i < J.ng; ++i) {
        const int32_t v = (int32_t)(gene_ic(J, i, genes[i]) + 0.5);
        h ^= (uint64_t)(int64_t)v + 0x9e3779b9ull + (h << 6) + (h >> 2);
    }
    return h;
}

// The signature set: open addressing in HBM; 0 marks an empty slot of the table, so the signature
// 0 is kept in gen[4] instead.
// Whether a signature is in the set (no insertion).
__device__ bool seen_contains(const GaJob& J, uint64_t h) {
    if (h == 0) return J.gen[4] != 0;
    unsigned long long i = mix64(h) & J.hmask;
    for (unsigned long long n = 0; n <= J.hmask; ++n, i = (i + 1) & J.hmask) {
        const uint64_t v = J.seen[i];
        if (v == h) return true;
        if (v == 0) return false;
    }
    return false;
}

// Inserts a signature the set does not hold, safe beside other threads inserting other
// signatures (the table's layout may differ from one-at-a-time insertion; membership does not).
__device__ void seen_insert_concurrent(const GaJob& J, uint64_t h) {
    if (h == 0) {
        J.gen[4] = 1;
        return;
    }
    unsigned long long i = mix64(h) & J.hmask;
    for (unsigned long long n = 0; n <= J.hmask; ++n, i = (i + 1) & J.hmask) {
        const unsigned long long prev = atomicCAS(reinterpret_cast<unsigned long long*>(J.seen) + i, 0ull,
                                                  (unsigned long long)h);
        if (prev == 0ull || prev == h) return;
    }
}

__device__ __forceinline__ int32_t uniform_gene(const GaJob& J, uint64_t i) {
    return (int32_t)(mix64(J.seed ^ mix64(0xFFFFFFFFull * 977 + i)) >> 33);
}

// Initial candidates c0 .. c0 + 2 npairs - 1: uniform genes in [0, 2^31) like the reference's
// RandomInt over MAX_RANDOM_VALUE; candidate c's gene q is draw c * ng + q. A rotamer gene is
// drawn only with its side chain's probability, else 0 (rotamer 0, the input conformation;
// generate_random_individual, LIB/gaboom.cpp:1875-1895), that chance being draw c * ng + q of
// stream kInitRotStream.
constexpr uint64_t kInitRotStream = 0xFFFFFFFEull;

// (the candidates first, first + stride, ... of the batch: the threads of a block, or of a grid)
__device__ void initial_candidates(const GaJob& J, long long c0, int npairs, int first, int stride) {
    const int ng = J.ng;
    for (int c = first; c < 2 * npairs; c += stride) {
        int32_t* g = J.cand + (size_t)c * ng;
        for (int q = 0; q < ng; ++q) {
            const uint64_t i = (uint64_t)(c0 + c) * ng + q;
            const float pr = J.gene_prob[q];
            g[q] = pr < 0.0f || uniform(J.seed, kInitRotStream, i) < (double)pr ? uniform_gene(J, i) : 0;
        }
        J.cand_sig[c] = signature(J, g);
    }
}

__global__ void __launch_bounds__(kGaThreads) ga_init_kernel(const GaJob* __restrict__ all, const int* __restrict__ run) {
    const GaJob& J = all[run[blockIdx.y]];
    initial_candidates(J, 0, min(J.ncand, J.gen[1]), blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// One pair of children: two roulette draws, optional adaptive probabilities, crossover with
// probability crossp, both children mutated bit by bit. draw() gives the next uniform in [0, 1)
// of the pair's stream, in the order the reference makes its draws.
template <typename Draw>
__device__ __forceinline__ void breed_pair_with(const GaJob& J, Draw&& draw, int32_t* john, int32_t* mary) {
    const int ng = J.ng;
    // fitness_stats (LIB/gaboom.cpp:818-840) of the population
    const double fit_max = J.fstat[1], fit_avg = J.fstat[2];
    const int pa = roulette(J, draw());
    const int pb = roulette(J, draw());
    const int a = J.ford[pa], b = J.ford[pb];
    double crossp = J.cross_rate, mutp = J.mut_rate;
    if (J.adaptive) {
        const double f1 = J.fit[pa], f2 = J.fit[pb];
        const double hi = f1 > f2 ? f1 : f2, lo = f1 > f2 ? f2 : f1;
        double denom = fit_max - fit_avg;
        if (denom < 1e-15) denom = 1e-15;   // GA_FITNESS_DENOM_FLOOR, LIB/ga_constants.h:38
        crossp = hi > fit_avg ? J.k[0] * (fit_max - hi) / denom : J.k[2];
        mutp = lo > fit_avg ? J.k[1] * (fit_max - lo) / denom : J.k[3];
    }
    const DrawThreshold mut = draw_threshold(mutp);
    int32_t* m = mary;
    for (int q = 0; q < ng; ++q) {
        john[q] = J.pop[(size_t)a * ng + q];
        m[q] = J.pop[(size_t)b * ng + q];
    }
    if (draw() < crossp) {
        // LIB/gaboom.cpp:2527-2598
        int gen_a = (int)(draw() * (double)ng);
        int gen_b = (int)(draw() * (double)ng);
        if (gen_a >= ng) gen_a = ng - 1;
        if (gen_b >= ng) gen_b = ng - 1;
        int pnt_a, pnt_b;
        if (J.intragenes) {
            pnt_a = (int)(draw() * 32.0);
            pnt_b = (int)(draw() * 32.0);
            if (gen_a > gen_b) {
                const int tg = gen_a, tp = pnt_a;
                gen_a = gen_b; pnt_a = pnt_b;
                gen_b = tg; pnt_b = tp;
            }
            if (gen_a == gen_b && pnt_a < pnt_b) {
                const int tp = pnt_b;
                pnt_b = pnt_a;
                pnt_a = tp;
            }
        } else {
            if (gen_a > gen_b) {
                const int tg = gen_a;
                gen_a = gen_b;
                gen_b = tg;
            }
            if (gen_a != gen_b) {
                pnt_a = draw() < 0.5 ? 32 : 0;
                pnt_b = draw() < 0.5 ? 32 : 0;
                if (gen_b - gen_a == 1 && pnt_a == 0 && pnt_b == 32) pnt_b = pnt_a;
            } else {
                pnt_a = 32;
                pnt_b = 0;
            }
        }
        for (int j = gen_a; j <= gen_b; ++j) {
            const int np = j == gen_a ? pnt_a : 32;
            // the reference's mask: 1, then np times optr |= optr << 1
            const uint32_t optr = np >= 31 ? 0xFFFFFFFFu : ((2u << np) - 1u);
            const uint32_t uj = (uint32_t)john[j], um = (uint32_t)m[j];
            john[j] = (int32_t)((uj & ~optr) | (um & optr));
            m[j] = (int32_t)((uj & optr) | (um & ~optr));
        }
        if (pnt_b > 0) {
            const int np = pnt_b - 1;
            const uint32_t optr = np >= 31 ? 0xFFFFFFFFu : ((2u << np) - 1u);
            const uint32_t uj = (uint32_t)john[gen_b], um = (uint32_t)m[gen_b];
            john[gen_b] = (int32_t)((uj & ~optr) | (um & optr));
            m[gen_b] = (int32_t)((uj & optr) | (um & ~optr));
        }
    }
    // mutate both children (LIB/gaboom.cpp:2620-2641): the genes before the rotamer genes, then
    // each rotamer gene with its side chain's probability (LIB/gaboom.cpp:944-966)
    for (int c = 0; c < 2; ++c) {
        int32_t* ch = c == 0 ? john : m;
        for (int q = 0; q < ng; ++q) {
            const float pr = J.gene_prob[q];
            if (pr >= 0.0f && !(draw() < (double)pr)) continue;
            uint32_t optr = 0u;
            for (int bit = 0; bit < 32; ++bit)
                if (draw.below(mut)) optr |= 1u << bit;
            ch[q] ^= (int32_t)optr;
        }
    }
}

// The draws of one pair: its counter-based stream.
struct StreamDraws {
    uint64_t seed, st, d;
    __device__ __forceinline__ double operator()() { return uniform(seed, st, d++); }
    __device__ __forceinline__ bool below(const DrawThreshold& t) { return uniform_bits(seed, st, d++) < t.bits; }
};

// Pair k of the children of generation g + 1, from the generation's counter-based stream.
__device__ void breed_pair(const GaJob& J, int g, int k, int32_t* john, int32_t* mary) {
    const uint64_t st = ((uint64_t)(g + 1) << 32) + (uint64_t)k;   // streams of generation g + 1
    breed_pair_with(J, StreamDraws{J.seed, st, 0}, john, mary);
}

// Pairs k0 .. k0 + npairs - 1 of the running generation's children as candidates, with their
// signatures.
// (the pairs first, first + stride, ... of the batch: the threads of a block, or of a grid)
__device__ void bred_candidates(const GaJob& J, int g, long long k0, int npairs, int first, int stride) {
    const int ng = J.ng;
    for (int k = first; k < npairs; k += stride) {
        int32_t* john = J.cand + (size_t)(2 * k) * ng;
        int32_t* mary = john + ng;
        breed_pair(J, g, (int)(k0 + k), john, mary);
        J.cand_sig[2 * k] = signature(J, john);
        J.cand_sig[2 * k + 1] = signature(J, mary);
    }
}

__global__ void __launch_bounds__(kGaThreads) ga_breed_kernel(const GaJob* __restrict__ all, const int* __restrict__ run) {
    const GaJob& J = all[run[blockIdx.y]];
    bred_candidates(J, J.gen[0], 0, min(J.ncand, J.gen[1]), blockIdx.x * blockDim.x + threadIdx.x,
                    gridDim.x * blockDim.x);
}

// Blocks per job of the first candidate batch (pairs up to P + 8 with P <= 2048; one pair per thread).
constexpr int kGaBatchBlocks = (2048 + 8 + kGaThreads - 1) / kGaThreads;

constexpr int kGaMaxBatches = 16;   // candidate batches before duplicates are let through

// Acceptance in the reference's order (child 1, then child 2 of each pair, until the generation
// has nnew children; the initial population: P chromosomes): a candidate is taken unless its
// signature was seen before in the job, and taken signatures join the set. Walked one candidate
// at a time, candidate c is taken exactly when its signature is in neither the set the batch
// started from nor at an earlier candidate of the batch (an earlier copy joined the set or was in
// it), up to the candidate that completes the generation; candidates after it are not looked at.
// So the block decides all of a batch's candidates at once: the first occurrences by a sort of
// (signature, index) pairs in shared memory, the set by read-only probes, the cut by an ordered
// scan; then it copies the taken ones into place and inserts their signatures. When a batch runs
// out, the block breeds the next batch of pairs. After kGaMaxBatches batches candidates are taken
// as they come (counted in gen[2]), where the reference would loop until mutation finds new genes.
// gen[1] sizes the next generation's first batch from what this one used; gen[3] counts rejected
// candidates.
constexpr int kAcceptThreads = 1024;
constexpr int kAcceptSort = 8192;                  // >= 2 (P + 8) candidates with P <= 2048
constexpr size_t kAcceptSmem = (size_t)kAcceptSort * (sizeof(uint64_t) + sizeof(uint16_t)) + kAcceptSort;

template <bool kInitial>
__global__ void __launch_bounds__(kAcceptThreads) ga_accept_kernel(const GaJob* __restrict__ all, const int* __restrict__ run) {
    extern __shared__ __align__(16) unsigned char acc_smem[];
    uint64_t* skey = reinterpret_cast<uint64_t*>(acc_smem);
    uint16_t* sidx = reinterpret_cast<uint16_t*>(skey + kAcceptSort);
    uint8_t* take = reinterpret_cast<uint8_t*>(sidx + kAcceptSort);
    __shared__ int wsum[kAcceptThreads / 32];
    __shared__ int s_cut, s_taken, s_rej;
    const GaJob& J = all[run[blockIdx.x]];
    const int ng = J.ng, g = J.gen[0];
    const int need = kInitial ? J.P : J.nnew;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int npairs = min(J.ncand, J.gen[1]);
    long long base = 0;   // candidate index of the batch's first entry
    int i = 0, used = 0, forced = 0, rejected = 0;
    for (int batch = 0;; ++batch) {
        const bool force = !J.reject || batch >= kGaMaxBatches;
        const int ncb = 2 * npairs;
        // 1. which candidates would be taken (before the cut)
        if (force) {
            for (int c = tid; c < ncb; c += kAcceptThreads) take[c] = 1;
        } else {
            int n2 = 1;
            while (n2 < ncb) n2 <<= 1;
            for (int k = tid; k < n2; k += kAcceptThreads) {
                skey[k] = k < ncb ? J.cand_sig[k] : ~0ull;
                sidx[k] = (uint16_t)k;
            }
            __syncthreads();
            for (int len = 2; len <= n2; len <<= 1)
                for (int j = len >> 1; j > 0; j >>= 1) {
                    for (int k = tid; k < n2; k += kAcceptThreads) {
                        const int l = k ^ j;
                        if (l > k) {
                            const bool up = (k & len) == 0;
                            const uint64_t ka = skey[k], kb = skey[l];
                            const bool gt = ka > kb || (ka == kb && sidx[k] > sidx[l]);
                            if (gt == up) {
                                skey[k] = kb;
                                skey[l] = ka;
                                const uint16_t t = sidx[k];
                                sidx[k] = sidx[l];
                                sidx[l] = t;
                            }
                        }
                    }
                    __syncthreads();
                }
            for (int k = tid; k < n2; k += kAcceptThreads) {
                const int c = sidx[k];
                if (c >= ncb) continue;
                const bool first = k == 0 || skey[k] != skey[k - 1];
                take[c] = first && !seen_contains(J, skey[k]) ? 1 : 0;
            }
        }
        __syncthreads();
        // 2. the cut: the candidate that takes the generation to `need`, by an ordered scan over
        // contiguous runs of candidates per thread
        const int per = (ncb + kAcceptThreads - 1) / kAcceptThreads;
        const int c0 = tid * per, c1 = min(ncb, c0 + per);
        int cnt = 0;
        for (int c = c0; c < c1; ++c) cnt += take[c];
        int inc = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31) wsum[warp] = inc;
        if (tid == 0) {
            s_cut = ncb;
            s_taken = 0;
            s_rej = 0;
        }
        __syncthreads();
        int wbase = 0;
        for (int w = 0; w < warp; ++w) wbase += wsum[w];
        const int left = need - i;
        int rank = wbase + inc - cnt;   // taken candidates before c0
        for (int c = c0; c < c1; ++c)
            if (take[c]) {
                if (rank == left - 1) s_cut = c;   // (one thread holds the cut, if any)
                ++rank;
            }
        __syncthreads();
        const int cut = s_cut;                  // last candidate looked at (ncb: none)
        // 3. copy the taken candidates up to the cut into place, insert their signatures, count
        int my_taken = 0, my_rej = 0;
        rank = wbase + inc - cnt;
        for (int c = c0; c < c1 && c <= cut; ++c) {
            if (c >= ncb) break;
            if (take[c]) {
                const int slot = i + rank;
                for (int q = 0; q < ng; ++q) J.child[(size_t)slot * ng + q] = J.cand[(size_t)c * ng + q];
                if (!force) seen_insert_concurrent(J, J.cand_sig[c]);
                ++rank;
                ++my_taken;
            } else {
                ++my_rej;
            }
        }
        if (my_taken) atomicAdd(&s_taken, my_taken);
        if (my_rej) atomicAdd(&s_rej, my_rej);
        __syncthreads();
        const int taken = s_taken;
        if (J.reject && force) forced += taken;
        rejected += s_rej;
        i += taken;
        used = (int)(base + cut + 1);
        const bool done = i == need;
        __syncthreads();
        if (done) break;
        base += 2 * npairs;
        npairs = J.ncand;
        if (kInitial) initial_candidates(J, base, npairs, threadIdx.x, blockDim.x);
        else bred_candidates(J, g, base >> 1, npairs, threadIdx.x, blockDim.x);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        int next;
        if (kInitial) {
            next = (J.nnew + 1) / 2 + J.nnew / 16 + 8;
        } else {
            const int pairs = (used + 1) / 2;
            next = pairs + pairs / 4 + 8;
        }
        J.gen[1] = min(J.ncand, next);
        J.gen[2] += forced;
        J.gen[3] += rejected;
    }
}

// Selection. kInitial: the evaluated initial population becomes generation 0. Otherwise the
// replacement: BOOM merges the P parents and nnew children, STEADY keeps the best P - nnew
// parents with the children in the places of the worst (child i at place P - 1 - i); the merged
// set is sorted by energy, the best P kept, saved as the generation's snapshot, and the
// generation counter advanced.
template <bool kInitial>
__global__ void __launch_bounds__(kGaSortThreads) ga_select_kernel(GaJob* __restrict__ all, const int* __restrict__ run) {
    __shared__ uint64_t key[kGaMaxSort];
    __shared__ int idx[kGaMaxSort];
    GaJob& J = all[run[blockIdx.x]];
    const int P = J.P, ng = J.ng, nnew = J.nnew;
    const int g = J.gen[0];
    int32_t* const pop = J.pop;
    int32_t* const nxt = J.pop_next;
    double* const pe = J.pop_e;
    double* const nxt_e = J.pop_e_next;
    // entries: parents [0, np_), then children; idx >= np_ names a child
    const int np_ = kInitial ? 0 : (J.steady ? P - nnew : P);
    const int m = kInitial ? P : np_ + nnew;
    int n = 1;
    while (n < m) n <<= 1;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double e = INFINITY;
        int id = i;
        if (i < m) {
            // STEADY: the place P-1-c holds child c
            const int c = kInitial ? i : (J.steady ? (P - 1 - i) : (i - np_));
            e = i < np_ ? pe[i] : J.child_cf[c].evalue;
            if (e != e) e = INFINITY;   // a NaN energy sorts last
            id = i;
        }
        key[i] = order_key(e);
        idx[i] = id;
    }
    __syncthreads();
    bitonic_sort(key, idx, n);
    // the new population, and (after a generation) its snapshot for the ensemble
    int32_t* const sg = kInitial ? nullptr : J.snap + (size_t)g * P * ng;
    double* const se = kInitial ? nullptr : J.snap_e + (size_t)g * P;
    for (int t = threadIdx.x; t < P * ng; t += blockDim.x) {
        const int r = t / ng, q = t - r * ng;
        const int src = idx[r];
        const int c = kInitial ? src : (J.steady ? (P - 1 - src) : (src - np_));
        const int32_t v = src < np_ ? pop[(size_t)src * ng + q] : J.child[(size_t)c * ng + q];
        nxt[t] = v;
        if (!kInitial) sg[t] = v;
    }
    for (int r = threadIdx.x; r < P; r += blockDim.x) {
        const int src = idx[r];
        const int c = kInitial ? src : (J.steady ? (P - 1 - src) : (src - np_));
        double e = src < np_ ? pe[src] : J.child_cf[c].evalue;
        if (e != e) e = INFINITY;
        nxt_e[r] = e;
        if (!kInitial) se[r] = e;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        J.pop = nxt;
        J.pop_next = pop;
        J.pop_e = nxt_e;
        J.pop_e_next = pe;
        if (!kInitial) J.gen[0] = g + 1;
    }
}

// ICs of the (new) population, clamped into the gene limits as eval_chromosome leaves them in
// the genes (LIB/gaboom.cpp:1845-1866), for the niche counts.
__global__ void __launch_bounds__(kGaThreads) ga_decode_kernel(const GaJob* __restrict__ all, const int* __restrict__ run) {
    const GaJob& J = all[run[blockIdx.y]];
    if (J.fitness == kFitLinear) return;
    const int n = J.P * J.ng;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int q = t % J.ng;
        double v = gene_ic(J, q, J.pop[t]);
        if (v > J.gene_max[q]) v = J.gene_max[q];
        else if (v < J.gene_min[q]) v = J.gene_min[q];
        J.pic[t] = v;
    }
}

constexpr int kNicheWarps = 8;
constexpr int kNicheBlocks = (2048 + kNicheWarps - 1) / kNicheWarps;

// Niche count of chromosome i: the sum over all j of 1 - (rmsp / sig_share)^alpha where rmsp
// (calc_rmsp, LIB/gaboom.cpp:2874-2885: root mean square of the IC differences) is within
// sig_share (LIB/gaboom.cpp:1652-1661). One warp per i: the lanes form the terms of 32 j's at a
// time, and the sum takes them in j order (a pair beyond sig_share adds 0, which changes no sum
// of these non-negative terms), so every count is the one a thread walking j in order forms.
__global__ void __launch_bounds__(kNicheWarps * 32) ga_niche_kernel(const GaJob* __restrict__ all, const int* __restrict__ run) {
    const GaJob& J = all[run[blockIdx.y]];
    const int i = blockIdx.x * kNicheWarps + (int)(threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (J.fitness == kFitLinear || i >= J.P) return;
    const int ng = J.ng, P = J.P;
    const double* xi = J.pic + (size_t)i * ng;
    const double sig = J.sig_share, alpha = J.share_alpha;
    double s = 0.0;
    for (int j0 = 0; j0 < P; j0 += 32) {
        const int j = j0 + lane;
        double term = 0.0;
        if (j < P) {
            const double* xj = J.pic + (size_t)j * ng;
            double acc = 0.0;
            for (int q = 0; q < ng; ++q) {
                const double dq = xi[q] - xj[q];
                acc += dq * dq;
            }
            const double r = sqrt(acc / (double)ng);
            if (r <= sig) term = 1.0 - (alpha == 1.0 ? r / sig : pow(r / sig, alpha));
        }
        const int m = P - j0 < 32 ? P - j0 : 32;
        for (int k = 0; k < m; ++k) s += __shfl_sync(0xffffffffu, term, k);
    }
    if (lane == 0) J.share[i] = s;
}

// Running sums of the fitness in roulette order (roullete_wheel's walk, LIB/gaboom.cpp:1158-1186)
// and fitness_stats' total, maximum and mean (LIB/gaboom.cpp:818-840), in order.
__device__ void fitness_sums(const GaJob& J, const double* fit, int P) {
    // (fitness_stats' total adds the same terms in the same order as the running sum: one sum;
    // the largest value, the first of equal ones, is found on the order keys, off the
    // double-precision pipe)
    double cum = 0.0;
    uint64_t mk = order_key(fit[0]);
    int mi = 0;
#pragma unroll 8
    for (int i = 0; i < P; ++i) {
        const double f = fit[i];
        cum += f;
        J.fcum[i] = cum;
        const uint64_t k = order_key(f);
        const bool nan = ((uint64_t)__double_as_longlong(f) << 1) > (0x7FF0000000000000ull << 1);
        if (k > mk && !nan) {   // (a NaN never compares greater)
            mk = k;
            mi = i;
        }
    }
    J.fstat[0] = cum;
    J.fstat[1] = fit[mi];
    J.fstat[2] = cum / (double)P;
}

// Fitness of the population (sorted by energy), the roulette order, running sums and
// fitness_stats. kInitial: the initial population, walked in energy order whatever the model.
template <bool kInitial>
__global__ void __launch_bounds__(kGaSortThreads) ga_fitness_kernel(const GaJob* __restrict__ all, const int* __restrict__ run) {
    // P <= kGaMaxSort / 2: the fitness, the sort keys (then the sorted fitness) and the order
    __shared__ double fval[kGaMaxSort / 2];
    __shared__ uint64_t key[kGaMaxSort / 2];
    __shared__ int idx[kGaMaxSort / 2];
    const GaJob& J = all[run[blockIdx.x]];
    const int P = J.P, model = J.fitness;
    const bool rank_only = model == kFitLinear || (model == kFitSmfree && !(J.beta > 0.0));
    double e0 = J.pop_e[0];
    if (!isfinite(e0)) e0 = 0.0;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        double f = (double)(P - i);
        if (!rank_only) {
            if (model == kFitPshare) {
                f = f / J.share[i];
            } else {
                // SMFREE (LIB/gaboom.cpp:1666-1736): the Boltzmann weight over the largest one
                // (that of the lowest energy)
                const double e = J.pop_e[i];
                const double bw = isfinite(e) && isfinite(J.pop_e[0]) ? exp(-J.beta * (e - e0)) : 0.0;
                const double blended = (1.0 - J.ent_w) * (f / (double)P) + J.ent_w * bw;
                f = blended * (double)P / J.share[i];
            }
        }
        fval[i] = f;
        idx[i] = i;
    }
    __syncthreads();
    const bool sorted = !kInitial && model == kFitPshare;
    if (sorted) {
        // QuickSort by fitness, descending (LIB/gaboom.cpp:499); equal fitness keeps energy order
        int n = 1;
        while (n < P) n <<= 1;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            key[i] = i < P ? order_key(-fval[i]) : order_key(INFINITY);
            idx[i] = i;
        }
        __syncthreads();
        bitonic_sort(key, idx, n);
    }
    double* const fs = reinterpret_cast<double*>(key);   // the fitness in roulette order
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const double f = fval[sorted ? idx[i] : i];
        fs[i] = f;
        J.fit[i] = f;
        J.ford[i] = idx[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) fitness_sums(J, fs, P);
}

void launch_ga_fitness(const GaJob* all, const int* run, int n_jobs, bool initial, cudaStream_t st) {
    ga_decode_kernel<<<dim3(8, n_jobs), kGaThreads, 0, st>>>(all, run);
    ga_niche_kernel<<<dim3(kNicheBlocks, n_jobs), kNicheWarps * 32, 0, st>>>(all, run);
    if (initial) ga_fitness_kernel<true><<<n_jobs, kGaSortThreads, 0, st>>>(all, run);
    else ga_fitness_kernel<false><<<n_jobs, kGaSortThreads, 0, st>>>(all, run);
}

// The acceptance kernels' shared memory (beyond the default 48 KB), allowed once per device.
static void accept_smem_attribute() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
    static bool done[64] = {false};
    if (done[dev]) return;
    cudaFuncSetAttribute(ga_accept_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kAcceptSmem);
    cudaFuncSetAttribute(ga_accept_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kAcceptSmem);
    done[dev] = true;
}

void launch_ga_init(const GaJob* all, const int* run, int n_jobs, cudaStream_t st) {
    ga_init_kernel<<<dim3(2 * kGaBatchBlocks, n_jobs), kGaThreads, 0, st>>>(all, run);
    accept_smem_attribute();
    ga_accept_kernel<true><<<n_jobs, kAcceptThreads, kAcceptSmem, st>>>(all, run);
}
void launch_ga_breed(const GaJob* all, const int* run, int n_jobs, cudaStream_t st) {
    ga_breed_kernel<<<dim3(kGaBatchBlocks, n_jobs), kGaThreads, 0, st>>>(all, run);
    accept_smem_attribute();
    ga_accept_kernel<false><<<n_jobs, kAcceptThreads, kAcceptSmem, st>>>(all, run);
}
// Breeding with the caller's draws (fxe_ga_breed_draws): J.fit and J.ford given, one block forms
// the running sums and fitness_stats, then one thread per pair breeds from its row of draws.
__global__ void ga_draws_stats_kernel(const GaJob* __restrict__ J) {
    if (threadIdx.x == 0 && blockIdx.x == 0) fitness_sums(*J, J->fit, J->P);
}

__global__ void __launch_bounds__(kGaThreads) ga_breed_draws_kernel(const GaJob* __restrict__ Jp, const double* __restrict__ draws,
                                                                    long long stride, int n_pairs, int* __restrict__ used) {
    const GaJob& J = *Jp;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_pairs) return;
    // the draws of one pair: its row of the caller's draws
    struct RowDraws {
        const double* row;
        long long stride, d;
        bool over;
        __device__ double operator()() {
            if (d >= stride) { over = true; return 0.0; }
            return row[d++];
        }
        __device__ bool below(const DrawThreshold& t) { return (*this)() < t.p; }
    } draw{draws + (size_t)k * stride, stride, 0, false};
    int32_t* john = J.child + (size_t)(2 * k) * J.ng;
    breed_pair_with(J, draw, john, john + J.ng);
    used[k] = draw.over ? -1 : (int)draw.d;
}

void launch_ga_breed_draws(const GaJob* J, const double* draws, long long stride, int n_pairs, int* used,
                           cudaStream_t st) {
    ga_draws_stats_kernel<<<1, 32, 0, st>>>(J);
    ga_breed_draws_kernel<<<(n_pairs + kGaThreads - 1) / kGaThreads, kGaThreads, 0, st>>>(J, draws, stride, n_pairs, used);
}

// Niche counts of a population whose ICs are given (fxe_ga_niche_counts): the generation's kernel
// on one job.
void launch_ga_niche(const GaJob* all, const int* run, cudaStream_t st) {
    ga_niche_kernel<<<dim3(kNicheBlocks, 1), kNicheWarps * 32, 0, st>>>(all, run);
}

void launch_ga_select(GaJob* all, const int* run, int n_jobs, bool initial, cudaStream_t st) {
    if (initial) ga_select_kernel<true><<<n_jobs, kGaSortThreads, 0, st>>>(all, run);
    else ga_select_kernel<false><<<n_jobs, kGaSortThreads, 0, st>>>(all, run);
}

}  // namespace fxe
