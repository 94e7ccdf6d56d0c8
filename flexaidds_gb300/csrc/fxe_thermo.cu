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

__device__ __forceinline__ void lse_push(LseState& st, double lw, double e) {
    if (lw > st.m) {
        const double sc = st.m == -INFINITY ? 0.0 : exp(st.m - lw);
        st.s = st.s * sc + 1.0;
        st.e1 = st.e1 * sc + e;
        st.e2 = st.e2 * sc + e * e;
        st.m = lw;
    } else {
        const double w = exp(lw - st.m);
        st.s += w;
        st.e1 += w * e;
        st.e2 += w * e * e;
    }
}

__device__ __forceinline__ LseState lse_merge(const LseState& a, const LseState& b) {
    if (b.m == -INFINITY) return a;
    if (a.m == -INFINITY) return b;
    const double M = fmax(a.m, b.m);
    const double fa = exp(a.m - M), fb = exp(b.m - M);
    return {M, a.s * fa + b.s * fb, a.e1 * fa + b.e1 * fb, a.e2 * fa + b.e2 * fb};
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
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        LseState other{__shfl_xor_sync(0xffffffffu, st.m, o), __shfl_xor_sync(0xffffffffu, st.s, o),
                       __shfl_xor_sync(0xffffffffu, st.e1, o), __shfl_xor_sync(0xffffffffu, st.e2, o)};
        st = lse_merge(st, other);
    }
    __shared__ LseState ws[kThermoThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = st;
    __syncthreads();
    if (threadIdx.x == 0) {
        LseState t = ws[0];
        for (int w = 1; w < kThermoThreads / 32; ++w) t = lse_merge(t, ws[w]);
        part[blockIdx.x] = {t.m, t.s, t.e1, t.e2};
    }
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

constexpr long kFixedPerBlock = (long)kThermoThreads * FXE_THERMO_FIXED_PER_THREAD;

// One partial per block; every slot a call reads is written by that call first, so nothing
// here needs to start at zero.
static __device__ __align__(256) LsePart g_fixed_part[FXE_THERMO_FIXED_MAX_BLOCKS];

cudaError_t fixed_scratch_address(LsePart** p) {
    return cudaGetSymbolAddress(reinterpret_cast<void**>(p), g_fixed_part);
}

__global__ void __launch_bounds__(kThermoThreads)
thermo_fixed_partial_kernel(const double* __restrict__ e, const int32_t* __restrict__ mult, long n,
                            double beta, LsePart* __restrict__ part) {
    LseState st{-INFINITY, 0.0, 0.0, 0.0};
    const long lo = (long)blockIdx.x * kFixedPerBlock;
    const long hi = lo + kFixedPerBlock < n ? lo + kFixedPerBlock : n;
    for (long i = lo + threadIdx.x; i < hi; i += kThermoThreads) {
        const double ei = e[i];
        const double lw = (mult ? log((double)mult[i]) : 0.0) - beta * ei;
        lse_push(st, lw, ei);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        LseState other{__shfl_xor_sync(0xffffffffu, st.m, o), __shfl_xor_sync(0xffffffffu, st.s, o),
                       __shfl_xor_sync(0xffffffffu, st.e1, o), __shfl_xor_sync(0xffffffffu, st.e2, o)};
        st = lse_merge(st, other);
    }
    __shared__ LseState ws[kThermoThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = st;
    __syncthreads();
    if (threadIdx.x == 0) {
        LseState t = ws[0];
        for (int w = 1; w < kThermoThreads / 32; ++w) t = lse_merge(t, ws[w]);
        part[blockIdx.x] = {t.m, t.s, t.e1, t.e2};
    }
}

// One block merges the partials and writes the record (the host merge of thermo_finish, done
// as a tree).
__global__ void __launch_bounds__(kThermoThreads)
thermo_fixed_finish_kernel(const LsePart* __restrict__ part, int nb, double T, fxe_thermo* __restrict__ out) {
    LseState st{-INFINITY, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nb; b += kThermoThreads) {
        const LsePart q = part[b];
        st = lse_merge(st, LseState{q.m, q.s, q.e1, q.e2});
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        LseState other{__shfl_xor_sync(0xffffffffu, st.m, o), __shfl_xor_sync(0xffffffffu, st.s, o),
                       __shfl_xor_sync(0xffffffffu, st.e1, o), __shfl_xor_sync(0xffffffffu, st.e2, o)};
        st = lse_merge(st, other);
    }
    __shared__ LseState ws[kThermoThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = st;
    __syncthreads();
    if (threadIdx.x == 0) {
        LseState t = ws[0];
        for (int w = 1; w < kThermoThreads / 32; ++w) t = lse_merge(t, ws[w]);
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

void launch_thermo_fixed(const double* e, const int32_t* mult, long n, double beta, double T,
                         LsePart* scratch, fxe_thermo* d_out, cudaStream_t st) {
    const int nb = (int)((n + kFixedPerBlock - 1) / kFixedPerBlock);
    thermo_fixed_partial_kernel<<<nb, kThermoThreads, 0, st>>>(e, mult, n, beta, scratch);
    thermo_fixed_finish_kernel<<<1, kThermoThreads, 0, st>>>(scratch, nb, T, d_out);
}

}  // namespace fxe
