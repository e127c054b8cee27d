// Batched solver engine: one thread block ("team") per work item, a work item
// being K right-hand sides of one system advanced in lockstep. Teams never wait
// on each other, so the launch needs no co-residency and every phase barrier is
// a block barrier. Each team runs a complete solve:
//
//   FP64 defect correction (outer):  r = b - A x in FP64, stop on ||r|| / ||b||
//   inner PCG (T = float: mixed mode, T = double: FP64 mode) on A c = r / ||r||,
//   with the reference's multicolor SSOR sweeps (ConjugateGradientSolverCSR_Rainbow,
//   solver/sparsesolver.cpp:1002-1335) or no preconditioner (plain CG, :26-201),
//   then x += ||r|| c.
//
// Matrix layout: SELL-32 ("sliced ELL") over the color-permuted rows. A slice is 32
// consecutive rows of one color; its entries are stored column-major in three
// blocks [L | E | U] (colors lower / equal / higher than the row's), each padded to
// the slice's longest row with zero entries. A warp owns a slice, a thread owns a
// row: loads of column indices and values are fully coalesced, no cross-lane
// reduction is needed, and the per-row epilogue runs on all lanes at once.
// Vectors of a team are interleaved [row][K] so one gather fetches the K values
// of a column in a single 8/16/32-byte load.
#include <cmath>
#include <cstdio>

#include "feec_batched.h"
#include "feec_device.cuh"

namespace feec {

namespace {

// L2 eviction priorities: every team of a batch streams the same matrix, while each
// team's vectors are private and touched once per phase. Matrix loads carry an
// evict_last cache policy so the shared operator stays in L2; row-local vector
// traffic uses streaming (evict-first) loads and stores.
__device__ __forceinline__ unsigned long long l2_keep_policy() {
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ int ld_keep(const int* a, unsigned long long pol) {
    int v;
    asm volatile("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ float ld_keep(const float* a, unsigned long long pol) {
    float v;
    asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ double ld_keep(const double* a, unsigned long long pol) {
    double v;
    asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(a), "l"(pol));
    return v;
}

template <typename T, int K> struct Vec;
template <> struct Vec<float, 1> { using t = float; };
template <> struct Vec<float, 2> { using t = float2; };
template <> struct Vec<float, 4> { using t = float4; };
template <> struct Vec<double, 1> { using t = double; };
template <> struct Vec<double, 2> { using t = double2; };

template <typename T, int K>
__device__ __forceinline__ void load_k(const T* p, T (&v)[K]) {
    if constexpr (K == 1) {
        v[0] = p[0];
    } else if constexpr (K == 2) {
        const typename Vec<T, 2>::t u = *reinterpret_cast<const typename Vec<T, 2>::t*>(p);
        v[0] = u.x; v[1] = u.y;
    } else if constexpr (K == 4 && sizeof(T) == 4) {
        const float4 u = *reinterpret_cast<const float4*>(p);
        v[0] = u.x; v[1] = u.y; v[2] = u.z; v[3] = u.w;
    } else {
        #pragma unroll
        for (int j = 0; j < K; j += 2) {
            const double2 u = *reinterpret_cast<const double2*>(p + j);
            v[j] = u.x; v[j + 1] = u.y;
        }
    }
}

// Accumulate sum_k val[k] * X[col[k]] over one column-major block of a slice.
// Memory-level parallelism: a chunk of CH column indices and values is loaded
// first (all independent, coalesced across the warp), then the CH gathers are
// issued together, then the FMAs run; padded slots are predicated off.
template <typename T, int K>
struct Chunk { static constexpr int value = (K >= 4) ? 8 : 16; };

template <typename T, typename TV, int K>
__device__ __forceinline__ void block_dot(const int* __restrict__ sci, const TV* __restrict__ sval, long long off,
                                          int len, int lane, const T* X, T (&s)[K]) {
    constexpr int CH = Chunk<T, K>::value;
    const unsigned long long pol = l2_keep_policy();
    for (int k0 = 0; k0 < len; k0 += CH) {
        int c[CH]; T v[CH];
        #pragma unroll
        for (int u = 0; u < CH; u++) {
            const bool ok = k0 + u < len;
            const long long p = off + (long long)(k0 + u) * 32 + lane;
            c[u] = ok ? ld_keep(&sci[p], pol) : -1;
            v[u] = ok ? (T)ld_keep(&sval[p], pol) : T(0);
        }
        T xv[CH][K];
        #pragma unroll
        for (int u = 0; u < CH; u++) {
            if (c[u] >= 0) {
                load_k<T, K>(X + (long long)c[u] * K, xv[u]);
            } else {
                #pragma unroll
                for (int j = 0; j < K; j++) xv[u][j] = T(0);
            }
        }
        #pragma unroll
        for (int u = 0; u < CH; u++)
            #pragma unroll
            for (int j = 0; j < K; j++) s[j] = fma(v[u], xv[u][j], s[j]);
    }
}

// Team-wide (block) deterministic sum of NV accumulators, result broadcast to all threads.
template <typename T, int NV>
__device__ __forceinline__ void team_sum(typename AccT<T>::type (&v)[NV], double (&out)[NV]) {
    __shared__ double s_out[NV];
    block_reduce<T, NV>(v);
    if (threadIdx.x == 0)
        #pragma unroll
        for (int k = 0; k < NV; k++) s_out[k] = AccT<T>::value(v[k]);
    __syncthreads();
    #pragma unroll
    for (int k = 0; k < NV; k++) out[k] = s_out[k];
    __syncthreads();
}

template <typename T>
__device__ __forceinline__ const T* sel_val(const SellView& S);
template <> __device__ __forceinline__ const float* sel_val<float>(const SellView& S) { return S.val32; }
template <> __device__ __forceinline__ const double* sel_val<double>(const SellView& S) { return S.val64; }
template <typename T>
__device__ __forceinline__ const T* sel_wd(const SellView& S);
template <> __device__ __forceinline__ const float* sel_wd<float>(const SellView& S) { return S.wd32; }
template <> __device__ __forceinline__ const double* sel_wd<double>(const SellView& S) { return S.wd64; }
template <typename T>
__device__ __forceinline__ const T* sel_sd(const SellView& S);
template <> __device__ __forceinline__ const float* sel_sd<float>(const SellView& S) { return S.sd32; }
template <> __device__ __forceinline__ const double* sel_sd<double>(const SellView& S) { return S.sd64; }

struct SliceMeta {
    int row0, nrow;
    int4 len;
    long long off;
};

__device__ __forceinline__ SliceMeta load_meta(const SellView& S, int sl) {
    SliceMeta m;
    m.row0 = __ldg(&S.slice_row0[sl]);
    m.nrow = __ldg(&S.slice_nrow[sl]);
    m.len = __ldg(&S.slice_len[sl]);
    m.off = __ldg(&S.slice_off[sl]);
    return m;
}

// Warp-strided loop over slices [s0, s1): the metadata of a warp's next slice is
// loaded while the current one is processed, so a slice costs two dependent
// memory round trips (its entries, then the gathers) instead of three.
template <typename F>
__device__ __forceinline__ void for_slices(const SellView& S, int s0, int s1, F&& body) {
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int sl = s0 + warp;
    SliceMeta cur{};
    if (sl < s1) cur = load_meta(S, sl);
    for (; sl < s1; sl += nwarps) {
        SliceMeta nxt{};
        if (sl + nwarps < s1) nxt = load_meta(S, sl + nwarps);
        body(cur);
        cur = nxt;
    }
}

template <typename T, int K>
__device__ __forceinline__ void load_k_stream(const T* p, T (&v)[K]) {
    if constexpr (K == 1) {
        v[0] = __ldcs(p);
    } else if constexpr (K == 2) {
        const typename Vec<T, 2>::t u = __ldcs(reinterpret_cast<const typename Vec<T, 2>::t*>(p));
        v[0] = u.x; v[1] = u.y;
    } else if constexpr (K == 4 && sizeof(T) == 4) {
        const float4 u = __ldcs(reinterpret_cast<const float4*>(p));
        v[0] = u.x; v[1] = u.y; v[2] = u.z; v[3] = u.w;
    } else {
        #pragma unroll
        for (int j = 0; j < K; j += 2) {
            const double2 u = __ldcs(reinterpret_cast<const double2*>(p + j));
            v[j] = u.x; v[j + 1] = u.y;
        }
    }
}

template <typename T, int K>
__device__ __forceinline__ void load_row(const T* v, int row, bool act, T (&out)[K]) {
    if (act) {
        load_k_stream<T, K>(v + (long long)row * K, out);
    } else {
        #pragma unroll
        for (int j = 0; j < K; j++) out[j] = T(0);
    }
}

template <typename T, int K>
__device__ __forceinline__ void store_row(T* v, int row, const T (&in)[K]) {
    T* p = v + (long long)row * K;
    if constexpr (K == 1) {
        __stcs(p, in[0]);
    } else if constexpr (K == 2) {
        typename Vec<T, 2>::t u; u.x = in[0]; u.y = in[1];
        __stcs(reinterpret_cast<typename Vec<T, 2>::t*>(p), u);
    } else if constexpr (K == 4 && sizeof(T) == 4) {
        __stcs(reinterpret_cast<float4*>(p), make_float4(in[0], in[1], in[2], in[3]));
    } else {
        #pragma unroll
        for (int j = 0; j < K; j += 2) __stcs(reinterpret_cast<double2*>(p + j), make_double2(in[j], in[j + 1]));
    }
}

// One team solves work item `it` completely.
template <typename T, int K, bool RAINBOW>
__device__ void team_solve(const BatchArgs& args, const BatchItem& it) {
    using AT = AccT<T>;
    using Acc = typename AT::type;
    const SellView S = args.systems[it.system];
    const int n = S.n;
    const int lane = threadIdx.x & 31;
    const int kk = it.nrhs;                       // active columns (<= K)
    const T* val = sel_val<T>(S);
    const T* wd = sel_wd<T>(S);
    const T* sd = sel_sd<T>(S);
    double* xp = it.xp; double* bp = it.bp; double* r64 = it.r64;
    T* r = (T*)it.r; T* d = (T*)it.d; T* z = (T*)it.z; T* m = (T*)it.m; T* q = (T*)it.q; T* c = (T*)it.c;
    __shared__ double s_scal[4][K];
    __shared__ int s_flag;

    // gather caller vectors into the permuted, interleaved layout; ||b||^2
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int o = __ldg(&S.perm[i]);
        #pragma unroll
        for (int j = 0; j < K; j++) {
            bp[(long long)i * K + j] = j < kk ? it.b[j][o] : 0.0;
            xp[(long long)i * K + j] = j < kk ? it.x[j][o] : 0.0;
        }
    }
    double bnorm2[K];
    {
        double a2[K];
        #pragma unroll
        for (int j = 0; j < K; j++) a2[j] = 0.0;
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            #pragma unroll
            for (int j = 0; j < K; j++) { const double v = bp[(long long)i * K + j]; a2[j] += v * v; }
        team_sum<double, K>(a2, bnorm2);
    }

    int done[K], iters[K], outer_cnt[K], status[K];
    double relres[K];
    #pragma unroll
    for (int j = 0; j < K; j++) { done[j] = j >= kk; iters[j] = 0; outer_cnt[j] = 0; status[j] = FEEC_MAXITER; relres[j] = -1.0; }

    for (int outer = 0; outer < args.max_outer; outer++) {
        // ---- FP64 true residual r64 = b - A x and its norm ----
        __syncthreads();
        double rn2[K];
        {
            double a2[K];
            #pragma unroll
            for (int j = 0; j < K; j++) a2[j] = 0.0;
            for_slices(S, 0, S.nslices, [&](const SliceMeta& M) {
                const int row = M.row0 + lane;
                const bool act = lane < M.nrow;
                double bv[K];
                load_row<double, K>(bp, row, act, bv);
                double sum[K];
                #pragma unroll
                for (int j = 0; j < K; j++) sum[j] = 0.0;
                block_dot<double, double, K>(S.ci, S.val64, M.off, M.len.x + M.len.y + M.len.z, lane, xp, sum);
                if (act) {
                    double rv[K];
                    #pragma unroll
                    for (int j = 0; j < K; j++) { rv[j] = bv[j] - sum[j]; a2[j] += rv[j] * rv[j]; }
                    store_row<double, K>(r64, row, rv);
                }
            });
            team_sum<double, K>(a2, rn2);
        }
        // stop tests per column (thread 0 decides, broadcast)
        if (threadIdx.x == 0) {
            int all = 1;
            for (int j = 0; j < K; j++) {
                if (j < kk) {
                    const double bn = sqrt(bnorm2[j]);
                    const double rn = sqrt(rn2[j]);
                    if (!done[j]) {
                        if (!(rn == rn)) { done[j] = 1; status[j] = FEEC_BREAKDOWN; }
                        else if (rn <= args.precision * bn) { done[j] = 1; status[j] = FEEC_OK; }
                        else if (iters[j] >= args.max_iter) { done[j] = 1; status[j] = FEEC_MAXITER; }
                    }
                    relres[j] = bn > 0.0 ? rn / bn : 0.0;
                    // inner target: the reduction still needed (with margin), never below eta
                    const double need = args.inner_margin * args.precision * bn / (rn > 0.0 ? rn : 1.0);
                    s_scal[0][j] = done[j] ? 0.0 : (rn > 0.0 ? 1.0 / rn : 0.0);
                    s_scal[1][j] = done[j] ? 0.0 : rn;
                    const double eta = need > args.inner_eta ? need : args.inner_eta;
                    s_scal[2][j] = eta * eta;
                } else {
                    s_scal[0][j] = 0.0; s_scal[1][j] = 0.0; s_scal[2][j] = 0.0;
                }
                all = all && done[j];
            }
            s_flag = all;
        }
        __syncthreads();
        // thread 0 decided; every other thread reads the decision (s_scal[1] == 0 <=> done)
        if (threadIdx.x != 0) {
            #pragma unroll
            for (int j = 0; j < K; j++) done[j] = s_scal[1][j] == 0.0;
        }
        if (s_flag) break;
        T inv[K];
        double rnorm[K], eta2d[K];
        #pragma unroll
        for (int j = 0; j < K; j++) { inv[j] = (T)s_scal[0][j]; rnorm[j] = s_scal[1][j]; eta2d[j] = s_scal[2][j]; }
        __syncthreads();

        // ---- inner solve: A c = r64 / ||r64|| in T; restart with c = 0, r = rin ----
        Acc arr[K], azr[K];
        #pragma unroll
        for (int j = 0; j < K; j++) { arr[j] = AT::zero(); azr[j] = AT::zero(); }
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            #pragma unroll
            for (int j = 0; j < K; j++) {
                const long long p = (long long)i * K + j;
                const T rv = (T)(r64[p] * (double)inv[j]);
                r[p] = rv; c[p] = T(0); m[p] = T(0); z[p] = T(0); q[p] = T(0);
                if constexpr (!RAINBOW) { d[p] = rv; azr[j] = AT::add(azr[j], rv * rv); } else { d[p] = T(0); }
                arr[j] = AT::add(arr[j], rv * rv);
            }
        }
        __syncthreads();
        if constexpr (RAINBOW) {
            for (int col = 0; col < S.ncolors; col++) {              // forward sweep
                for_slices(S, __ldg(&S.color_slice[col]), __ldg(&S.color_slice[col + 1]), [&](const SliceMeta& M) {
                    const int row = M.row0 + lane;
                    const bool act = lane < M.nrow;
                    const T w = act ? __ldg(&wd[row]) : T(0);
                    T rv[K];
                    load_row<T, K>(r, row, act, rv);
                    T sum[K];
                    #pragma unroll
                    for (int j = 0; j < K; j++) sum[j] = T(0);
                    block_dot<T, T, K>(S.ci, val, M.off, M.len.x, lane, m, sum);
                    if (act && w != T(0)) {
                        T mv[K];
                        #pragma unroll
                        for (int j = 0; j < K; j++) mv[j] = (rv[j] - sum[j]) * w;
                        store_row<T, K>(m, row, mv);
                    }
                });
                __syncthreads();
            }
            for (int col = S.ncolors - 1; col >= 0; col--) {         // scale + backward sweep
                for_slices(S, __ldg(&S.color_slice[col]), __ldg(&S.color_slice[col + 1]), [&](const SliceMeta& M) {
                    const int row = M.row0 + lane;
                    const bool act = lane < M.nrow;
                    const T w = act ? __ldg(&wd[row]) : T(0);
                    const T sdv = act ? __ldg(&sd[row]) : T(0);
                    T mv[K], rv[K];
                    load_row<T, K>(m, row, act, mv);
                    load_row<T, K>(r, row, act, rv);
                    T sum[K];
                    #pragma unroll
                    for (int j = 0; j < K; j++) sum[j] = T(0);
                    block_dot<T, T, K>(S.ci, val, M.off + 32ll * (M.len.x + M.len.y), M.len.z, lane, z, sum);
                    if (act && w != T(0)) {
                        T zv[K];
                        #pragma unroll
                        for (int j = 0; j < K; j++) {
                            mv[j] = mv[j] * sdv;
                            zv[j] = (mv[j] - sum[j]) * w;
                            azr[j] = AT::add(azr[j], zv[j] * rv[j]);
                        }
                        store_row<T, K>(m, row, mv);
                        store_row<T, K>(z, row, zv);
                        store_row<T, K>(d, row, zv);
                    }
                });
                __syncthreads();
            }
        }
        double zr[K], rr[K];
        {
            Acc both[2 * K];
            #pragma unroll
            for (int j = 0; j < K; j++) { both[j] = azr[j]; both[K + j] = arr[j]; }
            double o[2 * K];
            team_sum<T, 2 * K>(both, o);
            #pragma unroll
            for (int j = 0; j < K; j++) { zr[j] = o[j]; rr[j] = o[K + j]; }
        }
        int active[K];
        #pragma unroll
        for (int j = 0; j < K; j++) active[j] = !done[j];
        while (true) {
            // per-column stop on the recursive residual of the inner system
            int any = 0;
            #pragma unroll
            for (int j = 0; j < K; j++) {
                if (active[j] && (rr[j] < eta2d[j] || iters[j] >= args.max_iter)) active[j] = 0;
                any |= active[j];
            }
            if (!any) break;
            // q = A d (full rows), d.q
            Acc adq[K];
            #pragma unroll
            for (int j = 0; j < K; j++) adq[j] = AT::zero();
            for_slices(S, 0, S.nslices, [&](const SliceMeta& M) {
                const int row = M.row0 + lane;
                const bool act = lane < M.nrow;
                const bool skip = RAINBOW && (!act || __ldg(&wd[row]) == T(0));
                T dv[K];
                load_row<T, K>(d, row, act, dv);
                T sum[K];
                #pragma unroll
                for (int j = 0; j < K; j++) sum[j] = T(0);
                block_dot<T, T, K>(S.ci, val, M.off, M.len.x + M.len.y + M.len.z, lane, d, sum);
                if (act) {
                    T qv[K];
                    #pragma unroll
                    for (int j = 0; j < K; j++) {
                        qv[j] = skip ? T(0) : sum[j];
                        adq[j] = AT::add(adq[j], dv[j] * qv[j]);
                    }
                    store_row<T, K>(q, row, qv);
                }
            });
            double dq[K];
            team_sum<T, K>(adq, dq);
            T alpha[K];
            #pragma unroll
            for (int j = 0; j < K; j++) {
                alpha[j] = T(0);
                if (active[j]) {
                    if (!(dq[j] > 0.0) || !(zr[j] >= 0.0) || !isfinite(dq[j]) || !isfinite(zr[j])) active[j] = 0;
                    else alpha[j] = (T)(zr[j] / dq[j]);
                }
            }
            #pragma unroll
            for (int j = 0; j < K; j++) { arr[j] = AT::zero(); azr[j] = AT::zero(); }
            if constexpr (RAINBOW) {
                for (int col = 0; col < S.ncolors; col++) {
                    for_slices(S, __ldg(&S.color_slice[col]), __ldg(&S.color_slice[col + 1]), [&](const SliceMeta& M) {
                        const int row = M.row0 + lane;
                        const bool act = lane < M.nrow;
                        const T w = act ? __ldg(&wd[row]) : T(0);
                        T rv[K], qv[K], dv[K], cv[K];
                        load_row<T, K>(r, row, act, rv);
                        load_row<T, K>(q, row, act, qv);
                        load_row<T, K>(d, row, act, dv);
                        load_row<T, K>(c, row, act, cv);
                        T sum[K];
                        #pragma unroll
                        for (int j = 0; j < K; j++) sum[j] = T(0);
                        block_dot<T, T, K>(S.ci, val, M.off, M.len.x, lane, m, sum);
                        if (act && w != T(0)) {
                            T mv[K];
                            #pragma unroll
                            for (int j = 0; j < K; j++) {
                                cv[j] += alpha[j] * dv[j];
                                rv[j] = rv[j] - alpha[j] * qv[j];
                                arr[j] = AT::add(arr[j], rv[j] * rv[j]);
                                mv[j] = (rv[j] - sum[j]) * w;
                            }
                            store_row<T, K>(c, row, cv);
                            store_row<T, K>(r, row, rv);
                            store_row<T, K>(m, row, mv);
                        }
                    });
                    __syncthreads();
                }
                for (int col = S.ncolors - 1; col >= 0; col--) {
                    for_slices(S, __ldg(&S.color_slice[col]), __ldg(&S.color_slice[col + 1]), [&](const SliceMeta& M) {
                        const int row = M.row0 + lane;
                        const bool act = lane < M.nrow;
                        const T w = act ? __ldg(&wd[row]) : T(0);
                        const T sdv = act ? __ldg(&sd[row]) : T(0);
                        T mv[K], rv[K];
                        load_row<T, K>(m, row, act, mv);
                        load_row<T, K>(r, row, act, rv);
                        T sum[K];
                        #pragma unroll
                        for (int j = 0; j < K; j++) sum[j] = T(0);
                        block_dot<T, T, K>(S.ci, val, M.off + 32ll * (M.len.x + M.len.y), M.len.z, lane, z, sum);
                        if (act && w != T(0)) {
                            T zv[K];
                            #pragma unroll
                            for (int j = 0; j < K; j++) {
                                mv[j] = mv[j] * sdv;
                                zv[j] = (mv[j] - sum[j]) * w;
                                azr[j] = AT::add(azr[j], zv[j] * rv[j]);
                            }
                            store_row<T, K>(m, row, mv);
                            store_row<T, K>(z, row, zv);
                        }
                    });
                    __syncthreads();
                }
            } else {
                for (int i = threadIdx.x; i < n; i += blockDim.x)
                    #pragma unroll
                    for (int j = 0; j < K; j++) {
                        const long long p = (long long)i * K + j;
                        c[p] += alpha[j] * d[p];
                        const T rv = r[p] - alpha[j] * q[p];
                        r[p] = rv;
                        arr[j] = AT::add(arr[j], rv * rv);
                        azr[j] = AT::add(azr[j], rv * rv);
                    }
            }
            double zr_new[K];
            {
                Acc both[2 * K];
                #pragma unroll
                for (int j = 0; j < K; j++) { both[j] = azr[j]; both[K + j] = arr[j]; }
                double o[2 * K];
                team_sum<T, 2 * K>(both, o);
                #pragma unroll
                for (int j = 0; j < K; j++) { zr_new[j] = o[j]; rr[j] = active[j] ? o[K + j] : rr[j]; }
            }
            T beta[K];
            #pragma unroll
            for (int j = 0; j < K; j++) {
                beta[j] = active[j] ? (T)(zr_new[j] / zr[j]) : T(0);
                if (active[j]) { zr[j] = zr_new[j]; iters[j]++; }
            }
            // d = z + beta d for the active columns (CG: z = r)
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                if (RAINBOW && __ldg(&wd[i]) == T(0)) continue;
                #pragma unroll
                for (int j = 0; j < K; j++) {
                    if (!active[j]) continue;
                    const long long p = (long long)i * K + j;
                    d[p] = (RAINBOW ? z[p] : r[p]) + beta[j] * d[p];
                }
            }
            __syncthreads();
        }
        // x += ||r|| c in FP64
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            #pragma unroll
            for (int j = 0; j < K; j++) {
                const long long p = (long long)i * K + j;
                if (!done[j]) xp[p] += rnorm[j] * (double)c[p];
            }
        #pragma unroll
        for (int j = 0; j < K; j++) if (!done[j]) outer_cnt[j]++;
    }
    // scatter x back to the caller's numbering and report
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int o = __ldg(&S.perm[i]);
        #pragma unroll
        for (int j = 0; j < K; j++)
            if (j < kk) it.x[j][o] = xp[(long long)i * K + j];
    }
    if (threadIdx.x == 0) {
        for (int j = 0; j < kk; j++) {
            const int slot = it.first_result + j;
            args.results[slot].status = done[j] ? status[j] : FEEC_MAXITER;
            args.results[slot].iterations = iters[j];
            args.results[slot].outer = outer_cnt[j];
            args.results[slot].relres = relres[j];
        }
    }
}

template <typename T, int K, bool RAINBOW, int THREADS>
__global__ void __launch_bounds__(THREADS) batched_solve_kernel(BatchArgs args) {
    __shared__ int s_item;
    while (true) {
        if (threadIdx.x == 0) s_item = atomicAdd(args.next_item, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= args.nitems) return;
        team_solve<T, K, RAINBOW>(args, args.items[item]);
    }
}

template <typename T, int K, bool RB>
const void* kfn(int threads) {
    if constexpr (sizeof(T) == 4) {
        if (threads == 128) return (const void*)batched_solve_kernel<T, K, RB, 128>;
        if (threads == 512) return (const void*)batched_solve_kernel<T, K, RB, 512>;
    }
    return (const void*)batched_solve_kernel<T, K, RB, 256>;
}

const void* pick(int is_float, int K, int rainbow, int threads) {
    if (is_float) {
        if (rainbow) return K == 1 ? kfn<float, 1, true>(threads) : K == 2 ? kfn<float, 2, true>(threads) : kfn<float, 4, true>(threads);
        return K == 1 ? kfn<float, 1, false>(threads) : K == 2 ? kfn<float, 2, false>(threads) : kfn<float, 4, false>(threads);
    }
    if (rainbow) return K == 1 ? kfn<double, 1, true>(threads) : kfn<double, 2, true>(threads);
    return K == 1 ? kfn<double, 1, false>(threads) : kfn<double, 2, false>(threads);
}

}  // namespace

int batched_max_k(int is_float) { return is_float ? 4 : 2; }

int batched_team_threads(int is_float, int requested) {
    if (!is_float) return 256;
    return (requested == 128 || requested == 512) ? requested : 256;
}

int batched_resident_teams(int is_float, int K, int rainbow, int threads) {
    threads = batched_team_threads(is_float, threads);
    const void* fn = pick(is_float, K, rainbow, threads);
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, 0);
    return sms * (per > 0 ? per : 1);
}

cudaError_t launch_batched(const BatchArgs& args, int is_float, int K, int rainbow, int threads, int teams, cudaStream_t s) {
    threads = batched_team_threads(is_float, threads);
    const void* fn = pick(is_float, K, rainbow, threads);
    if (teams <= 0) teams = batched_resident_teams(is_float, K, rainbow, threads);
    if (teams > args.nitems) teams = args.nitems;
    if (teams <= 0) return cudaSuccess;
    BatchArgs copy = args;
    void* kargs[] = {&copy};
    note_launch();
    return cudaLaunchKernel(fn, dim3(teams), dim3(threads), kargs, 0, s);
}

}  // namespace feec
