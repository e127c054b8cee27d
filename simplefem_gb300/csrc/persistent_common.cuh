// Building blocks shared by the persistent (one cooperative launch per solve) Krylov
// kernels: row-group iteration, lane-split segment dot products, per-block partial
// sums and the status epilogue.
#pragma once
#include <type_traits>

#include "feec_device.cuh"
#include "feec_internal.h"

namespace feec {

constexpr int kThreads = 512;
constexpr int kLongLanes = 16;   // lanes per row for the long rows of a multicolor phase (split_rows)
constexpr double kMachineEpsilon = 2.220446049250313080847263336181640625e-16;  // base/base.hpp:123

// Iterate rows [lo, hi) with LANES lanes per row; the loop trip count is
// uniform across each warp so the shuffles inside `body` see all 32 lanes.
#define FEEC_FOR_ROW_GROUPS(lo, hi, row, active)                                                   \
    for (int _base = (lo) + (int)((blockIdx.x * blockDim.x + threadIdx.x) / 32) * (32 / LANES);    \
         _base < (hi); _base += (int)(gridDim.x * blockDim.x / 32) * (32 / LANES))                  \
        for (int row = _base + (int)((threadIdx.x & 31) / LANES), _once = 1; _once; _once = 0)      \
            for (bool active = row < (hi); _once; _once = 0)

// Accumulates s += v[j] * x[ci[j]] for j = j0, j0 + LANES, ... < hi in that order, four
// strides at a time: the four column indices and values are requested together, then the
// four gathers, so a long row costs two memory round trips per four strides instead of
// two per stride. The terms and their order are those of the one-stride loop.
template <typename T, int LANES>
__device__ __forceinline__ T seg_accumulate(const int* __restrict__ ci, const T* __restrict__ v, const T* x, int j0,
                                            int hi, T s) {
    for (int j = j0; j < hi; j += 4 * LANES) {
        int c[4];
        T w[4];
        #pragma unroll
        for (int u = 0; u < 4; u++) {
            const int k = j + u * LANES;
            c[u] = k < hi ? __ldg(&ci[k]) : -1;
            w[u] = k < hi ? __ldg(&v[k]) : T(0);
        }
        T g[4];
        #pragma unroll
        for (int u = 0; u < 4; u++) g[u] = c[u] >= 0 ? x[c[u]] : T(0);
        #pragma unroll
        for (int u = 0; u < 4; u++)
            if (c[u] >= 0) s = fma(w[u], g[u], s);
    }
    return s;
}

template <typename T, int LANES>
__device__ __forceinline__ T seg_dot(const int* __restrict__ ci, const T* __restrict__ v, const T* x, int lo, int hi,
                                     int lane) {
    T s = seg_accumulate<T, LANES>(ci, v, x, lo + lane, hi, T(0));
    #pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off, LANES);
    return s;
}

template <typename T>
__device__ __forceinline__ void write_partials(double* dst, typename AccT<T>::type v0) {
    typename AccT<T>::type v[1] = {v0};
    block_reduce<T, 1>(v);
    if (threadIdx.x == 0) dst[blockIdx.x] = AccT<T>::value(v[0]);
}

template <typename T>
__device__ __forceinline__ void write_partials2(double* dst, typename AccT<T>::type v0, typename AccT<T>::type v1) {
    typename AccT<T>::type v[2] = {v0, v1};
    block_reduce<T, 2>(v);
    if (threadIdx.x == 0) {
        dst[2 * blockIdx.x + 0] = AccT<T>::value(v[0]);
        dst[2 * blockIdx.x + 1] = AccT<T>::value(v[1]);
    }
}

// Rows [lo, hi) of a multicolor phase whose rows are sorted longest first, [lo, sp) being
// the long ones: the long rows get LL lanes each (the first warps of the grid), the rest LS
// lanes each (the warps after them), so that no row group walks more than a few strides
// of its row. A phase lasts as long as its slowest row group: with LS lanes for every row,
// the longest rows of a color (65 entries on 3D P2) took several dependent rounds of index
// loads and gathers while the other warps waited at the barrier. body(lanes, row, active,
// lane in group) is called with std::integral_constant lanes, uniformly across each warp.
template <int LS, int LL, typename F>
__device__ __forceinline__ void split_rows(int lo, int sp, int hi, F&& body) {
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) / 32);
    const int nwarps = (int)(gridDim.x * blockDim.x / 32);
    const int wl = (sp - lo + (32 / LL) - 1) / (32 / LL);   // warps the long rows take
    for (int w = warp; w < wl; w += nwarps) {
        const int i = lo + w * (32 / LL) + (int)((threadIdx.x & 31) / LL);
        body(std::integral_constant<int, LL>{}, i, i < sp, (int)(threadIdx.x & (LL - 1)));
    }
    int w = warp - wl % nwarps;
    if (w < 0) w += nwarps;
    for (; sp + w * (32 / LS) < hi; w += nwarps) {
        const int i = sp + w * (32 / LS) + (int)((threadIdx.x & 31) / LS);
        body(std::integral_constant<int, LS>{}, i, i < hi, (int)(threadIdx.x & (LS - 1)));
    }
}

__device__ __forceinline__ void finish(DeviceStatus* st, int status, int K, double fv, double av) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicCAS(&st->status, FEEC_OK, status);
        st->iterations = K;
        st->final_value = fv;
        st->aux_value = av;
    }
}

}  // namespace feec
