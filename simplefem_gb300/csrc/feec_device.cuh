// Device-side building blocks shared by the solver kernels: bounded grid
// barrier for co-resident (cooperatively launched) grids, deterministic block
// and grid reductions, compensated FP32 accumulation, and sub-warp CSR row dots.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "feec_gpu.h"

namespace feec {

// ---------------------------------------------------------------------------
// Status words written by kernels (kept in device memory, read by the host).
// ---------------------------------------------------------------------------
struct DeviceStatus {
    int status;          // FEEC_OK or an error/termination code
    int iterations;      // K as the reference counts it
    int timeout_site;    // barrier index at which a wait gave up (diagnostics)
    int abort;           // set by any block that gives up; every block then leaves
    double final_value;  // r.r (CG) or z.r (PCG) at exit
    double aux_value;    // d.Ad at a breakdown, or the inner r.r for the FP32 solver
    unsigned long long barrier;  // monotonically increasing grid-barrier counter
    double extra[4];
};

// Spin limits: every wait gives up after this many polls or this much time.
constexpr unsigned long long kSpinLimit = 1ull << 27;
constexpr unsigned long long kWaitNanos = 4000000000ull;  // 4 s

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_volatile_i32(const int* p) {
    int v;
    asm volatile("ld.volatile.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// One thread waits until the counter st->barrier reaches `target`. Gives up after
// `limit_ns` (or kSpinLimit polls), or when another block has given up: it then sets
// the abort flag, FEEC_TIMEOUT and the site, and returns false.
__device__ __forceinline__ bool wait_counter(DeviceStatus* st, unsigned long long target, int site,
                                             unsigned long long limit_ns) {
    unsigned long long spins = 0, t0 = 0;
    while (ld_acquire_u64(&st->barrier) < target) {
        ++spins;
        if ((spins & 255ull) == 0) {
            if (ld_volatile_i32(&st->abort)) return false;
            const unsigned long long t = globaltimer_ns();
            if (t0 == 0) t0 = t;
            if (spins > kSpinLimit || t - t0 > limit_ns) {
                atomicExch(&st->abort, 1);
                atomicCAS(&st->status, FEEC_OK, FEEC_TIMEOUT);
                atomicExch(&st->timeout_site, site);
                return false;
            }
        }
        if (spins > 32) __nanosleep(32);
    }
    return true;
}

// Arrival at a grid barrier: a release reduction (no return value to wait for) that
// publishes every write the block made before it (the preceding __syncthreads orders the
// other threads' writes before this thread's release).
__device__ __forceinline__ void arrive_release(unsigned long long* p) {
    asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(p) : "memory");
}

// Grid-wide barrier for a cooperatively launched grid. `epoch` is the number of
// barriers this block has passed (identical in every block). Arrival is a release
// reduction and the wait an acquire load (wait_counter), so no separate fences are
// needed; the __syncthreads on either side carry the ordering to the block's other
// threads. Returns false if the wait gave up (time or poll limit) or another block gave
// up; the caller must then leave the kernel without touching shared state again.
__device__ __forceinline__ bool grid_barrier(DeviceStatus* st, unsigned long long& epoch, int site) {
    if (gridDim.x * gridDim.y == 1) {   // a one-block grid (small systems): the block barrier suffices
        __syncthreads();
        return true;
    }
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        epoch += 1;
        const unsigned long long target = epoch * (unsigned long long)(gridDim.x * gridDim.y);
        arrive_release(&st->barrier);
        s_ok = wait_counter(st, target, site, kWaitNanos) ? 1 : 0;
    }
    __syncthreads();
    return s_ok != 0;
}

// ---------------------------------------------------------------------------
// Accumulators: plain double for FP64, compensated (TwoSum) float pairs for FP32.
// ---------------------------------------------------------------------------
struct CompF {
    float s, c;
};

__device__ __forceinline__ CompF comp_add(CompF a, float v) {
    // Knuth TwoSum: s + e == a.s + v exactly
    const float s = a.s + v;
    const float bp = s - a.s;
    const float e = (a.s - (s - bp)) + (v - bp);
    return CompF{s, a.c + e};
}

__device__ __forceinline__ CompF comp_merge(CompF a, CompF b) {
    const float s = a.s + b.s;
    const float bp = s - a.s;
    const float e = (a.s - (s - bp)) + (b.s - bp);
    return CompF{s, a.c + b.c + e};
}

template <typename T> struct AccT;
template <> struct AccT<double> {
    using type = double;
    __device__ __forceinline__ static double zero() { return 0.0; }
    __device__ __forceinline__ static double add(double a, double v) { return a + v; }
    __device__ __forceinline__ static double merge(double a, double b) { return a + b; }
    __device__ __forceinline__ static double value(double a) { return a; }
    __device__ __forceinline__ static double shfl_xor(double a, int m) { return __shfl_xor_sync(0xffffffffu, a, m); }
};
template <> struct AccT<float> {
    using type = CompF;
    __device__ __forceinline__ static CompF zero() { return CompF{0.f, 0.f}; }
    __device__ __forceinline__ static CompF add(CompF a, float v) { return comp_add(a, v); }
    __device__ __forceinline__ static CompF merge(CompF a, CompF b) { return comp_merge(a, b); }
    __device__ __forceinline__ static double value(CompF a) { return (double)a.s + (double)a.c; }
    __device__ __forceinline__ static CompF shfl_xor(CompF a, int m) {
        return CompF{__shfl_xor_sync(0xffffffffu, a.s, m), __shfl_xor_sync(0xffffffffu, a.c, m)};
    }
};

// Deterministic block reduction of NV accumulators; result valid in thread 0.
// Fixed shuffle tree + fixed warp order: same inputs give the same bits.
template <typename T, int NV>
__device__ __forceinline__ void block_reduce(typename AccT<T>::type (&v)[NV]) {
    using A = AccT<T>;
    using Acc = typename A::type;
    __shared__ Acc s_part[32][NV];
    #pragma unroll
    for (int k = 0; k < NV; k++)
        #pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[k] = A::merge(v[k], A::shfl_xor(v[k], off));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0)
        #pragma unroll
        for (int k = 0; k < NV; k++) s_part[warp][k] = v[k];
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        #pragma unroll
        for (int k = 0; k < NV; k++) {
            Acc a = lane < nw ? s_part[lane][k] : A::zero();
            #pragma unroll
            for (int off = 16; off > 0; off >>= 1) a = A::merge(a, A::shfl_xor(a, off));
            v[k] = a;
        }
    }
}

// Sum of the per-block partials (written as doubles: NV per block, block-major)
// in a fixed order; every block obtains the same bits. Called after a barrier.
template <int NV>
__device__ __forceinline__ void grid_sum(const double* partials, double (&out)[NV]) {
    __shared__ double s_out[NV];
    const int nb = gridDim.x;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        #pragma unroll
        for (int k = 0; k < NV; k++) {
            double a = 0.0;
            for (int b = lane; b < nb; b += 32) a += __ldcg(&partials[(size_t)b * NV + k]);
            #pragma unroll
            for (int off = 16; off > 0; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
            if (lane == 0) s_out[k] = a;
        }
    }
    __syncthreads();
    #pragma unroll
    for (int k = 0; k < NV; k++) out[k] = s_out[k];
    __syncthreads();
}

// Compensated variant: partials hold (s, c) float pairs widened to double.
// Summing the widened pairs in double is exact enough for any grid size here.

// ---------------------------------------------------------------------------
// Row dot of CSR segment [lo, hi) with vector `x`, by a group of LANES lanes.
// Result is valid in every lane of the group.
// ---------------------------------------------------------------------------
template <typename T, int LANES>
__device__ __forceinline__ T row_dot(const int* __restrict__ ci, const T* __restrict__ v, const T* x,
                                     int lo, int hi, int lane) {
    T s = T(0);
    for (int j = lo + lane; j < hi; j += LANES) s = fma(__ldg(&v[j]), x[__ldg(&ci[j])], s);
    #pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off, LANES);
    return s;
}

}  // namespace feec
