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

// One partial per block, and after them one slot for the count of finished blocks; every slot a
// call reads is written (or, the count, cleared) by that call first, so nothing here needs to
// start at zero.
static __device__ __align__(256) LsePart g_fixed_part[FXE_THERMO_FIXED_MAX_BLOCKS + 1];

cudaError_t fixed_scratch_address(LsePart** p) {
    return cudaGetSymbolAddress(reinterpret_cast<void**>(p), g_fixed_part);
}

// The fixed-scratch reduction in one launch: each thread takes its energies four at a time (their
// log-weights' maximum rescales the thread's sums at most once, then four independent exps), the
// blocks merge max first and write their partials, and the last block to finish (a counter in
// the scratch, cleared before the launch) merges the partials and writes the record. Each block
// covers a contiguous run of per_block energies.
constexpr int kFixedChunk = 4;

__global__ void __launch_bounds__(kThermoThreads)
thermo_fixed_kernel(const double* __restrict__ e, const int32_t* __restrict__ mult, long n, long per_block,
                    double beta, double T, LsePart* __restrict__ part, unsigned* __restrict__ done,
                    fxe_thermo* __restrict__ out) {
    const long lo = (long)blockIdx.x * per_block;
    const long hi = lo + per_block < n ? lo + per_block : n;
    LseState st{-INFINITY, 0.0, 0.0, 0.0};
    #pragma unroll 1
    for (long i0 = lo + threadIdx.x; i0 < hi; i0 += (long)kFixedChunk * kThermoThreads) {
        double ev[kFixedChunk], lw[kFixedChunk];
        double m4 = -INFINITY;
#pragma unroll
        for (int j = 0; j < kFixedChunk; ++j) {
            const long i = i0 + (long)j * kThermoThreads;
            ev[j] = 0.0;
            lw[j] = -INFINITY;
            if (i < hi) {
                ev[j] = e[i];
                lw[j] = (mult ? log((double)mult[i]) : 0.0) - beta * ev[j];
                m4 = fmax(m4, lw[j]);
            }
        }
        if (m4 > st.m) {
            const double f = st.m == -INFINITY ? 0.0 : exp(st.m - m4);
            st.s *= f;
            st.e1 *= f;
            st.e2 *= f;
            st.m = m4;
        }
#pragma unroll
        for (int j = 0; j < kFixedChunk; ++j) {
            if (lw[j] == -INFINITY) continue;
            const double w = exp(lw[j] - st.m);
            st.s += w;
            st.e1 += w * ev[j];
            st.e2 += w * ev[j] * ev[j];
        }
    }
    const LseState t = block_merge(st);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = {t.m, t.s, t.e1, t.e2};
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the last block: every partial, rescaled to their largest maximum, then the block's
    const int nb = (int)gridDim.x;
    double mt = -INFINITY;
    for (int b = threadIdx.x; b < nb; b += kThermoThreads) mt = fmax(mt, ((volatile LsePart*)part)[b].m);
    LseState sp{mt, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nb; b += kThermoThreads) {
        const volatile LsePart* q = (volatile LsePart*)part + b;
        const double qm = q->m;
        if (qm == -INFINITY) continue;
        const double f = exp(qm - mt);
        sp.s += q->s * f;
        sp.e1 += q->e1 * f;
        sp.e2 += q->e2 * f;
    }
    const LseState r = block_merge(sp);
    if (threadIdx.x == 0) {
        const double kB = 0.001987206;  // LIB/statmech.h:26
        const double lnZ = r.m + log(r.s);
        const double Ea = r.e1 / r.s, E2 = r.e2 / r.s;
        const double kT = kB * T;
        const double var = E2 - Ea * Ea;
        fxe_thermo rec;
        rec.temperature = T;
        rec.log_Z = lnZ;
        rec.free_energy = -kT * lnZ;
        rec.mean_energy = Ea;
        rec.mean_energy_sq = E2;
        rec.heat_capacity = var / (kT * kT);
        rec.entropy = (Ea - rec.free_energy) / T;
        rec.std_energy = sqrt(var > 0.0 ? var : 0.0);
        *out = rec;
    }
}

// Blocks of the fixed-scratch pass: one chunk of four energies per thread when the partials allow
// it, within the FXE_THERMO_FIXED_MAX_BLOCKS partials.
void launch_thermo_fixed(const double* e, const int32_t* mult, long n, double beta, double T,
                         LsePart* scratch, fxe_thermo* d_out, cudaStream_t st) {
    long nb = (n + (long)kFixedChunk * kThermoThreads - 1) / ((long)kFixedChunk * kThermoThreads);
    if (nb > FXE_THERMO_FIXED_MAX_BLOCKS) nb = FXE_THERMO_FIXED_MAX_BLOCKS;
    if (nb < 1) nb = 1;
    long per_block = (n + nb - 1) / nb;
    if (per_block < 1) per_block = 1;
    nb = (n + per_block - 1) / per_block;
    if (nb < 1) nb = 1;
    unsigned* done = reinterpret_cast<unsigned*>(scratch + FXE_THERMO_FIXED_MAX_BLOCKS);
    cudaMemsetAsync(done, 0, sizeof(unsigned), st);
    thermo_fixed_kernel<<<(int)nb, kThermoThreads, 0, st>>>(e, mult, n, per_block, beta, T, scratch, done, d_out);
}

}  // namespace fxe
