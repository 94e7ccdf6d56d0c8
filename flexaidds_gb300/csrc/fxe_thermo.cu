// fxe_thermo.cu — FP64 canonical-ensemble reduction (StatMechEngine::compute,
// LIB/statmech.cpp:73-174, and boltzmann_weights, :178-201).
//
// One pass over the energies: every thread keeps an online log-sum-exp state
// (running max m of the log-weights lw = ln n - beta E, s = sum exp(lw - m), and the first and
// second energy moments weighted the same way); blocks merge their threads' states and write one
// partial each; the host merges the partials. This equals the reference's three passes
// (max-shifted log-sum-exp of LIB/UnifiedHardwareDispatch.cpp:800-843, then the moments with
// p = exp(lw - lnZ)) up to rounding, and reads each energy once.
#include <cmath>

#include "fxe_common.cuh"

namespace fxe {

constexpr int kThermoThreads = 256;

struct LseState {
    double m, s, e1, e2;
};

// One energy into the state. Both cases take exp(-|lw - m|): the rescale factor of the sums when
// lw is a new maximum, the weight of the energy otherwise; one exp per energy and no divergent
// exp between the lanes of a warp. (With no energy yet, m = -inf and the factor is exp(-inf) = 0.)
__device__ __forceinline__ void lse_push(LseState& st, double lw, double e) {
    const double d = lw - st.m;
    const double x = exp(-fabs(d));
    if (d > 0.0) {
        st.s = st.s * x + 1.0;
        st.e1 = st.e1 * x + e;
        st.e2 = st.e2 * x + e * e;
        st.m = lw;
    } else {
        st.s += x;
        st.e1 += x * e;
        st.e2 += x * e * e;
    }
}

// The block's states merged, max first: the block's maximum M by shuffles, then each thread's
// sums rescaled once by exp(m - M) and added up (one exp per thread instead of one per merge).
// Every thread of the block calls it; thread 0 gets the result.
__device__ LseState block_merge(const LseState& st) {
    __shared__ double wm[kThermoThreads / 32];
    __shared__ double ws[3][kThermoThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double m = st.m;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) wm[warp] = m;
    __syncthreads();
    double M = wm[0];
    for (int w = 1; w < kThermoThreads / 32; ++w) M = fmax(M, wm[w]);
    const double f = st.m == -INFINITY ? 0.0 : exp(st.m - M);
    double a = st.s * f, b = st.e1 * f, c = st.e2 * f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if (lane == 0) {
        ws[0][warp] = a;
        ws[1][warp] = b;
        ws[2][warp] = c;
    }
    __syncthreads();
    LseState t{M, 0.0, 0.0, 0.0};
    if (threadIdx.x == 0)
        for (int w = 0; w < kThermoThreads / 32; ++w) {
            t.s += ws[0][w];
            t.e1 += ws[1][w];
            t.e2 += ws[2][w];
        }
    return t;
}

__global__ void __launch_bounds__(kThermoThreads)
thermo_partial_kernel(const double* __restrict__ e, const int32_t* __restrict__ mult, long n,
                      double beta, LsePart* __restrict__ part) {
    LseState st{-INFINITY, 0.0, 0.0, 0.0};
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double ei = e[i];
        const double lw = (mult ? log((double)mult[i]) : 0.0) - beta * ei;
        lse_push(st, lw, ei);
    }
    const LseState t = block_merge(st);
    if (threadIdx.x == 0) part[blockIdx.x] = {t.m, t.s, t.e1, t.e2};
}

__global__ void thermo_weights_kernel(const double* __restrict__ e, const int32_t* __restrict__ mult,
                                      long n, double beta, double lnZ, double* __restrict__ w) {
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double lw = (mult ? log((double)mult[i]) : 0.0) - beta * e[i];
        w[i] = exp(lw - lnZ);
    }
}

int thermo_blocks(long n, int sms) {
    long b = (n + kThermoThreads - 1) / kThermoThreads;
    const long cap = (long)sms * 8;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

void launch_thermo_partial(const double* e, const int32_t* mult, long n, double beta, LsePart* part,
                           int blocks, cudaStream_t st) {
    thermo_partial_kernel<<<blocks, kThermoThreads, 0, st>>>(e, mult, n, beta, part);
}

void launch_thermo_weights(const double* e, const int32_t* mult, long n, double beta, double lnZ,
                           double* w, int blocks, cudaStream_t st) {
    thermo_weights_kernel<<<blocks, kThermoThreads, 0, st>>>(e, mult, n, beta, lnZ, w);
}

// Host merge of the block partials into the reference's Thermodynamics record.
void thermo_finish(const LsePart* part, int nb, double T, fxe_thermo* out) {
    const double kB = 0.001987206;  // LIB/statmech.h:26
    double M = -INFINITY;
    for (int b = 0; b < nb; ++b) M = part[b].m > M ? part[b].m : M;
    double s = 0.0, e1 = 0.0, e2 = 0.0;
    for (int b = 0; b < nb; ++b) {
        if (part[b].m == -INFINITY) continue;
        const double f = std::exp(part[b].m - M);
        s += part[b].s * f;
        e1 += part[b].e1 * f;
        e2 += part[b].e2 * f;
    }
    const double lnZ = M + std::log(s);
    const double Ea = e1 / s, E2 = e2 / s;
    const double kT = kB * T;
    const double var = E2 - Ea * Ea;
    out->temperature = T;
    out->log_Z = lnZ;
    out->free_energy = -kT * lnZ;
    out->mean_energy = Ea;
    out->mean_energy_sq = E2;
    out->heat_capacity = var / (kT * kT);
    out->entropy = (Ea - out->free_energy) / T;
    out->std_energy = std::sqrt(var > 0.0 ? var : 0.0);
}

}  // namespace fxe

// ------------------------------------------------------------------------------------------
// Fixed-scratch variant: the same reduction with the block partials in a file-scope device
// array and the merge on the device, for callers that may not allocate (see
// fxe_thermo_compute_device_fixed in include/fxe.h).
// ------------------------------------------------------------------------------------------
namespace fxe {

// One partial per block, and after them one slot for the maximum; every slot a call reads is
// written (or, the maximum, cleared) by that call first, so nothing here needs to start at zero.
static __device__ __align__(256) LsePart g_fixed_part[FXE_THERMO_FIXED_MAX_BLOCKS + 1];

// Order-preserving 64-bit key of a double (atomicMax on keys is a maximum on doubles; key 0 is
// below every number).
__device__ __forceinline__ unsigned long long order_key(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_order_key(unsigned long long k) {
    return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

cudaError_t fixed_scratch_address(LsePart** p) {
    return cudaGetSymbolAddress(reinterpret_cast<void**>(p), g_fixed_part);
}

// The block maximum of a double over all its threads (every thread calls it; all get it).
__device__ double block_max(double m) {
    __shared__ double wm[kThermoThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    double M = wm[0];
    for (int w = 1; w < kThermoThreads / 32; ++w) M = fmax(M, wm[w]);
    __syncthreads();
    return M;
}

// The fixed-scratch reduction runs max first, so that the pass with the exps has no chain between
// its energies: (1) the maximum log-weight M (each block's, into one slot by atomicMax on order
// keys; the slot is cleared before); (2) each block sums exp(lw - M) and its energy moments;
// (3) one block adds the blocks' sums. Each block covers a contiguous run of per_block energies.
__global__ void __launch_bounds__(kThermoThreads)
thermo_fixed_max_kernel(const double* __restrict__ e, const int32_t* __restrict__ mult, long n,
                        long per_block, double beta, unsigned long long* __restrict__ max_key) {
    const long lo = (long)blockIdx.x * per_block;
    const long hi = lo + per_block < n ? lo + per_block : n;
    double m = -INFINITY;
    for (long i = lo + threadIdx.x; i < hi; i += kThermoThreads)
        m = fmax(m, (mult ? log((double)mult[i]) : 0.0) - beta * e[i]);
    m = block_max(m);
    if (threadIdx.x == 0) atomicMax(max_key, order_key(m));
}

__global__ void __launch_bounds__(kThermoThreads)
thermo_fixed_sum_kernel(const double* __restrict__ e, const int32_t* __restrict__ mult, long n,
                        long per_block, double beta, const unsigned long long* __restrict__ max_key,
                        LsePart* __restrict__ part) {
    const double M = from_order_key(*max_key);
    const long lo = (long)blockIdx.x * per_block;
    const long hi = lo + per_block < n ? lo + per_block : n;
    LseState st{M, 0.0, 0.0, 0.0};
    for (long i = lo + threadIdx.x; i < hi; i += kThermoThreads) {
        const double ei = e[i];
        const double w = exp((mult ? log((double)mult[i]) : 0.0) - beta * ei - M);
        st.s += w;
        st.e1 += w * ei;
        st.e2 += w * ei * ei;
    }
    const LseState t = block_merge(st);
    if (threadIdx.x == 0) part[blockIdx.x] = {M, t.s, t.e1, t.e2};
}

// One block adds the blocks' sums (all relative to the same maximum) and writes the record.
__global__ void __launch_bounds__(kThermoThreads)
thermo_fixed_finish_kernel(const LsePart* __restrict__ part, int nb, double T, fxe_thermo* __restrict__ out) {
    LseState st{part[0].m, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nb; b += kThermoThreads) {
        const LsePart q = part[b];
        st.s += q.s;
        st.e1 += q.e1;
        st.e2 += q.e2;
    }
    const LseState t = block_merge(st);
    if (threadIdx.x == 0) {
        const double kB = 0.001987206;  // LIB/statmech.h:26
        const double lnZ = t.m + log(t.s);
        const double Ea = t.e1 / t.s, E2 = t.e2 / t.s;
        const double kT = kB * T;
        const double var = E2 - Ea * Ea;
        fxe_thermo r;
        r.temperature = T;
        r.log_Z = lnZ;
        r.free_energy = -kT * lnZ;
        r.mean_energy = Ea;
        r.mean_energy_sq = E2;
        r.heat_capacity = var / (kT * kT);
        r.entropy = (Ea - r.free_energy) / T;
        r.std_energy = sqrt(var > 0.0 ? var : 0.0);
        *out = r;
    }
}

// Blocks of the fixed-scratch passes: about four energies per thread, within the
// FXE_THERMO_FIXED_MAX_BLOCKS partials.
void launch_thermo_fixed(const double* e, const int32_t* mult, long n, double beta, double T,
                         LsePart* scratch, fxe_thermo* d_out, cudaStream_t st) {
    long nb = (n + 4 * kThermoThreads - 1) / (4 * kThermoThreads);
    if (nb > FXE_THERMO_FIXED_MAX_BLOCKS) nb = FXE_THERMO_FIXED_MAX_BLOCKS;
    if (nb < 1) nb = 1;
    long per_block = (n + nb - 1) / nb;
    if (per_block < 1) per_block = 1;
    nb = (n + per_block - 1) / per_block;
    if (nb < 1) nb = 1;
    unsigned long long* max_key = reinterpret_cast<unsigned long long*>(scratch + FXE_THERMO_FIXED_MAX_BLOCKS);
    cudaMemsetAsync(max_key, 0, sizeof(unsigned long long), st);
    thermo_fixed_max_kernel<<<(int)nb, kThermoThreads, 0, st>>>(e, mult, n, per_block, beta, max_key);
    thermo_fixed_sum_kernel<<<(int)nb, kThermoThreads, 0, st>>>(e, mult, n, per_block, beta, max_key, scratch);
    thermo_fixed_finish_kernel<<<1, kThermoThreads, 0, st>>>(scratch, (int)nb, T, d_out);
}

}  // namespace fxe
