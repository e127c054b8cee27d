// Device solver shared by the batched engine (one block per work item) and the
// cluster engine (one thread-block cluster per request, used by the serving loop):
// FP64 defect correction around an FP32 (or FP64) inner PCG with the reference's
// multicolor SSOR sweeps or no preconditioner, over a SELL-32 layout. The code is
// written once against a Team policy (BlockTeam / ClusterTeam).
#pragma once
#include <cmath>
#include <cstdio>

#include <cooperative_groups.h>

#include "feec_batched.h"
#include "feec_device.cuh"

namespace feec {
namespace team_solver {
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
    } else if constexpr (K % 4 == 0 && sizeof(T) == 4) {
        #pragma unroll
        for (int j = 0; j < K; j += 4) {
            const float4 u = *reinterpret_cast<const float4*>(p + j);
            v[j] = u.x; v[j + 1] = u.y; v[j + 2] = u.z; v[j + 3] = u.w;
        }
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
struct Chunk { static constexpr int value = sizeof(T) == 8 ? ((K >= 2) ? 2 : 4) : (K >= 8 ? 2 : ((K >= 4) ? 2 : 4)); };

template <typename T, typename TV, int CH>
__device__ __forceinline__ void load_entries(const int* __restrict__ sci, const TV* __restrict__ sval, long long off,
                                             int k0, int len, int lane, unsigned long long pol, int (&c)[CH],
                                             T (&v)[CH]) {
    #pragma unroll
    for (int u = 0; u < CH; u++) {
        const bool ok = k0 + u < len;
        const long long p = off + (long long)(k0 + u) * 32 + lane;
        c[u] = ok ? ld_keep(&sci[p], pol) : -1;
        v[u] = ok ? (T)ld_keep(&sval[p], pol) : T(0);
    }
}

// Software-pipelined over chunks of CH entries: the column indices and values of the
// next chunk are requested together with the gathers of the current one, so a chunk
// costs one memory round trip instead of two.
template <typename T, typename TV, int K>
__device__ __forceinline__ void block_dot(const int* __restrict__ sci, const TV* __restrict__ sval, long long off,
                                          int len, int lane, const T* X, T (&s)[K]) {
    constexpr int CH = Chunk<T, K>::value;
    const unsigned long long pol = l2_keep_policy();
    if (len <= 0) return;
    int c[CH]; T v[CH];
    load_entries<T, TV, CH>(sci, sval, off, 0, len, lane, pol, c, v);
    for (int k0 = 0; k0 < len; k0 += CH) {
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
        int cn[CH]; T vn[CH];
        load_entries<T, TV, CH>(sci, sval, off, k0 + CH, len, lane, pol, cn, vn);
        #pragma unroll
        for (int u = 0; u < CH; u++)
            #pragma unroll
            for (int j = 0; j < K; j++) s[j] = fma(v[u], xv[u][j], s[j]);
        #pragma unroll
        for (int u = 0; u < CH; u++) { c[u] = cn[u]; v[u] = vn[u]; }
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

// ---------------------------------------------------------------------------
// Team policies. A team is the set of threads that solves one work item together.
//   BlockTeam   — one thread block; phase barrier = __syncthreads.
//   ClusterTeam — a thread-block cluster (co-scheduled by the hardware on one GPC);
//                 phase barrier = cluster barrier (release/acquire at cluster scope),
//                 team sums read every block's partial through distributed shared
//                 memory in a fixed order, so every block obtains the same bits.
// Neither waits on anything outside its own co-scheduled threads.
// ---------------------------------------------------------------------------
struct BlockTeam {
    __device__ __forceinline__ int rank() const { return 0; }
    __device__ __forceinline__ int size() const { return 1; }
    __device__ __forceinline__ int tid() const { return threadIdx.x; }
    __device__ __forceinline__ int nthreads() const { return blockDim.x; }
    __device__ __forceinline__ void sync() { __syncthreads(); }
    template <typename T, int NV>
    __device__ __forceinline__ void sum(typename AccT<T>::type (&v)[NV], double (&out)[NV]) { team_sum<T, NV>(v, out); }
};

struct ClusterTeam {
    int r, sz, buf;
    __device__ ClusterTeam() : buf(0) {
        cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
        r = (int)cl.block_rank();
        sz = (int)cl.num_blocks();
    }
    __device__ __forceinline__ int rank() const { return r; }
    __device__ __forceinline__ int size() const { return sz; }
    __device__ __forceinline__ int tid() const { return r * blockDim.x + threadIdx.x; }
    __device__ __forceinline__ int nthreads() const { return sz * blockDim.x; }
    __device__ __forceinline__ void sync() { cooperative_groups::this_cluster().sync(); }
    template <typename T, int NV>
    __device__ __forceinline__ void sum(typename AccT<T>::type (&v)[NV], double (&out)[NV]) {
        __shared__ double s_part[2][NV];
        __shared__ double s_res[NV];
        block_reduce<T, NV>(v);
        if (threadIdx.x == 0)
            #pragma unroll
            for (int k = 0; k < NV; k++) s_part[buf][k] = AccT<T>::value(v[k]);
        cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
        cl.sync();
        if (threadIdx.x == 0) {
            double acc[NV];
            #pragma unroll
            for (int k = 0; k < NV; k++) acc[k] = 0.0;
            for (int q = 0; q < sz; q++) {
                const double* rp = cl.map_shared_rank(&s_part[buf][0], q);
                #pragma unroll
                for (int k = 0; k < NV; k++) acc[k] += rp[k];
            }
            #pragma unroll
            for (int k = 0; k < NV; k++) s_res[k] = acc[k];
        }
        __syncthreads();
        #pragma unroll
        for (int k = 0; k < NV; k++) out[k] = s_res[k];
        __syncthreads();
        buf ^= 1;   // the next sum writes the other slot; this one is reused two sums later
    }
};

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
template <typename Team, typename F>
__device__ __forceinline__ void for_slices(const Team& team, const SellView& S, int s0, int s1, F&& body) {
    const int warp = team.rank() * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int nwarps = team.size() * (blockDim.x >> 5);
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
    } else if constexpr (K % 4 == 0 && sizeof(T) == 4) {
        #pragma unroll
        for (int j = 0; j < K; j += 4) {
            const float4 u = __ldcs(reinterpret_cast<const float4*>(p + j));
            v[j] = u.x; v[j + 1] = u.y; v[j + 2] = u.z; v[j + 3] = u.w;
        }
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
    } else if constexpr (K % 4 == 0 && sizeof(T) == 4) {
        #pragma unroll
        for (int j = 0; j < K; j += 4)
            __stcs(reinterpret_cast<float4*>(p + j), make_float4(in[j], in[j + 1], in[j + 2], in[j + 3]));
    } else {
        #pragma unroll
        for (int j = 0; j < K; j += 2) __stcs(reinterpret_cast<double2*>(p + j), make_double2(in[j], in[j + 1]));
    }
}

// ---------------------------------------------------------------------------
// Slice streaming: each warp walks its slices of a phase; the metadata of its next
// slice is loaded while the current one is processed, the slice's own-row values
// (pre) are requested before its gathers, and the row epilogue (post) runs on all
// 32 lanes at once. Measured on GB300: staging the column/value stream through
// shared memory with cp.async was slower than these direct loads — the multicolor
// gathers, not the matrix stream, bound the sweeps.
// ---------------------------------------------------------------------------
inline int team_dynamic_smem(int) { return 0; }

enum { kBlockFull = 0, kBlockL = 1, kBlockU = 2 };

template <int WHICH>
__device__ __forceinline__ void block_range(const SliceMeta& M, long long& off, int& len) {
    if (WHICH == kBlockFull) { off = M.off; len = M.len.x + M.len.y + M.len.z; }
    else if (WHICH == kBlockL) { off = M.off; len = M.len.x; }
    else { off = M.off + 32ll * (M.len.x + M.len.y); len = M.len.z; }
}

// Per-row state carried from the prologue (own-row loads) to the epilogue of a slice.
template <typename U, int K>
struct RowState {
    int row;
    bool act;
    U w, sdv;
    U a[K], b[K], c[K], e[K];
};

template <typename U, typename TV, int K, int WHICH, typename Team, typename Pre, typename Post>
__device__ __forceinline__ void for_slices_dot(const Team& team, const SellView& S, int s0, int s1, const TV* val,
                                               const U* X, Pre&& pre, Post&& post) {
    const int lane = threadIdx.x & 31;
    for_slices(team, S, s0, s1, [&](const SliceMeta& M) {
        auto state = pre(M);
        long long off; int len;
        block_range<WHICH>(M, off, len);
        U sum[K];
        #pragma unroll
        for (int j = 0; j < K; j++) sum[j] = U(0);
        block_dot<U, TV, K>(S.ci, val, off, len, lane, X, sum);
        post(M, state, sum);
    });
}

// Per-column control state of a team, in shared memory: thread 0 of every block
// updates it from the team sums (all blocks of a cluster team compute the same values
// from the same sums) and the other threads read the few scalars a phase needs. Keeping
// the bookkeeping out of registers leaves them to the slice loops.
template <typename T, int K>
struct TeamControl {
    double bnorm2[K], relres[K], stall[K], rnorm[K], zr[K];
    double thr[K];       // the column's segment ends once zr < thr
    double amp[K];       // largest measured error-to-residual amplification of column j (0: none yet)
    int iters[K], outer[K], status[K];
    T alpha[K], beta[K], inv[K];
    int err_step;    // bit j: column j met the residual bar but not yet the error bar
    int done;        // bit j: column j finished (converged, failed or absent)
    int active;      // bit j: column j iterates in this segment
    int trig;        // bit j: column j asked for the residual replacement that ends the segment
    int all_done;
};

// ---------------------------------------------------------------------------
// Mixed precision: FP64 defect correction around FP32 inner solves. The FP64 solution x and
// true residual r64 = b - A x are kept beside the inner iteration, which runs in T (FP32 in
// mixed precision) on the residual equation scaled to unit norm, A c = r64 / ||r64||, from
// c = 0 with a fresh Krylov recurrence. A segment ends when the column's preconditioned
// residual measure z.r has fallen by the square of args.inner_eta or far enough for its
// target; the correction is added to x in FP64 (x += ||r64|| c) and the true residual is
// recomputed. (Reliable updates, keeping the direction across the replacement, gained 2.5 %
// here at 1,216 columns in lockstep — any column's replacement ends every column's
// segment — and are used by the whole-GPU single-system solver only.)
// ---------------------------------------------------------------------------

// Plain CG (ConjugateGradientSolverCSR, solver/sparsesolver.cpp:26-201) on the scaled
// residual equation: the restart is r = r64 / ||r64|| (z = r), c = 0, and d = 0, so the first
// d = r + beta d (beta = 0) is r.
template <typename T, int K, typename Team>
__device__ void cg_transform(Team& team, const SellView& S, TeamControl<T, K>& ctl, const double* r64, T* r, T* d,
                             T* c, double (&zr)[K]) {
    using AT = AccT<T>;
    using Acc = typename AT::type;
    const int n = S.n;
    Acc arr[K];
    #pragma unroll
    for (int j = 0; j < K; j++) arr[j] = AT::zero();
    T inv[K];
    #pragma unroll
    for (int j = 0; j < K; j++) inv[j] = ctl.inv[j];
    for (int i = team.tid(); i < n; i += team.nthreads()) {
        #pragma unroll
        for (int j = 0; j < K; j++) {
            const long long p = (long long)i * K + j;
            const T rv = (T)(r64[p] * (double)inv[j]);
            r[p] = rv; c[p] = T(0); d[p] = T(0);
            arr[j] = AT::add(arr[j], rv * rv);
        }
    }
    team.template sum<T, K>(arr, zr);
}

// One CG iteration for the active columns: d = r + beta d, q = A d, alpha = r.r / d.q,
// c += alpha d, r -= alpha q; the new r.r comes back in rr.
template <typename T, int K, typename Team>
__device__ void cg_iterate(Team& team, const SellView& S, TeamControl<T, K>& ctl, const T* val, T* r, T* d, T* q,
                           T* c, double (&rr)[K]) {
    using AT = AccT<T>;
    using Acc = typename AT::type;
    const int n = S.n;
    const int lane = threadIdx.x & 31;
    const bool leader = threadIdx.x == 0;
    {
        T beta[K];
        #pragma unroll
        for (int j = 0; j < K; j++) beta[j] = ctl.beta[j];
        for (int i = team.tid(); i < n; i += team.nthreads()) {
            T rv[K], dv[K];
            load_k_stream<T, K>(r + (long long)i * K, rv);
            load_k_stream<T, K>(d + (long long)i * K, dv);
            #pragma unroll
            for (int j = 0; j < K; j++) dv[j] = rv[j] + beta[j] * dv[j];
            store_row<T, K>(d, i, dv);
        }
    }
    team.sync();
    Acc adq[K];
    #pragma unroll
    for (int j = 0; j < K; j++) adq[j] = AT::zero();
    for_slices_dot<T, T, K, kBlockFull>(team, S, 0, S.nslices, val, d,
        [&](const SliceMeta& M) {
            RowState<T, K> p;
            p.row = M.row0 + lane; p.act = lane < M.nrow;
            load_row<T, K>(d, p.row, p.act, p.a);
            return p;
        },
        [&](const SliceMeta&, const RowState<T, K>& p, const T (&sum)[K]) {
            if (p.act) {
                #pragma unroll
                for (int j = 0; j < K; j++) adq[j] = AT::add(adq[j], p.a[j] * sum[j]);
                store_row<T, K>(q, p.row, sum);
            }
        });
    {
        double dq[K];
        team.template sum<T, K>(adq, dq);
        if (leader) {
            int act = ctl.active;
            for (int j = 0; j < K; j++) {
                T a = T(0);
                if (act >> j & 1) {
                    const double zr = ctl.zr[j];
                    if (!(dq[j] > 0.0) || !(zr >= 0.0) || !isfinite(dq[j]) || !isfinite(zr)) act &= ~(1 << j);
                    else a = (T)(zr / dq[j]);
                }
                ctl.alpha[j] = a;
            }
            ctl.active = act;
        }
    }
    __syncthreads();
    Acc arr[K];
    T alpha[K];
    #pragma unroll
    for (int j = 0; j < K; j++) { alpha[j] = ctl.alpha[j]; arr[j] = AT::zero(); }
    for (int i = team.tid(); i < n; i += team.nthreads())
        #pragma unroll
        for (int j = 0; j < K; j++) {
            const long long p = (long long)i * K + j;
            c[p] += alpha[j] * d[p];
            const T rv = r[p] - alpha[j] * q[p];
            r[p] = rv;
            arr[j] = AT::add(arr[j], rv * rv);
        }
    team.template sum<T, K>(arr, rr);
}

// Multicolor SSOR-PCG in Eisenstat's formulation
// (ConjugateGradientSolverCSR_Eisenstat_Rainbow, solver/sparsesolver.cpp:1338-1645): the
// same preconditioned iterates as the Rainbow solver (:1002-1335) in exact arithmetic, but
// an iteration is one backward and one forward sweep over the strict parts — no SpMV
// over full rows — so each stored entry is read and gathered once per iteration instead
// of twice. Vectors (interleaved [row][K]): r = L-solved residual, d = direction,
// m = technical (backward sweep), q = auxiliary (forward sweep), c = solution. z = S r is
// not stored: the backward sweep forms it from r and the row factor (one FP32 vector
// stream less per column and iteration).
// With sd = D (2 - w) / w, the reference's (2/w - 1) D equals sd. A direction update
// d = z + beta d runs inside the backward sweep (a row's d is read only by the row itself).

// The restart of a segment: auxiliary = r64 / ||r64||, r = L-solve of it, z = S r, d = z,
// c = 0. `init` (the first segment): every work vector starts at 0, so rows the sweeps skip
// (D == 0) hold 0 wherever a gather reads them.
template <typename T, int K, typename Team>
__device__ void eis_transform(Team& team, const SellView& S, TeamControl<T, K>& ctl, const T* val, const T* wd,
                              const T* sd, const double* r64, T* r, T* d, T* m, T* q, T* c, bool init,
                              double (&zr)[K]) {
    using AT = AccT<T>;
    using Acc = typename AT::type;
    const int n = S.n;
    const int lane = threadIdx.x & 31;
    {
        T inv[K];
        #pragma unroll
        for (int j = 0; j < K; j++) inv[j] = ctl.inv[j];
        for (int i = team.tid(); i < n; i += team.nthreads()) {
            #pragma unroll
            for (int j = 0; j < K; j++) {
                const long long p = (long long)i * K + j;
                q[p] = (T)(r64[p] * (double)inv[j]);
                c[p] = T(0);
                if (init) { r[p] = T(0); d[p] = T(0); m[p] = T(0); }
            }
        }
    }
    team.sync();
    Acc azr[K];
    #pragma unroll
    for (int j = 0; j < K; j++) azr[j] = AT::zero();
    for (int col = 0; col < S.ncolors; col++) {
        for_slices_dot<T, T, K, kBlockL>(team, S, __ldg(&S.color_slice[col]), __ldg(&S.color_slice[col + 1]), val, r,
            [&](const SliceMeta& M) {
                RowState<T, K> p;
                p.row = M.row0 + lane; p.act = lane < M.nrow;
                p.w = p.act ? __ldg(&wd[p.row]) : T(0);
                p.sdv = p.act ? __ldg(&sd[p.row]) : T(0);
                load_row<T, K>(q, p.row, p.act, p.a);
                return p;
            },
            [&](const SliceMeta&, const RowState<T, K>& p, const T (&sum)[K]) {
                if (p.act && p.w != T(0)) {
                    T rv[K], zv[K];
                    #pragma unroll
                    for (int j = 0; j < K; j++) {
                        rv[j] = (p.a[j] - sum[j]) * p.w;
                        zv[j] = rv[j] * p.sdv;
                        azr[j] = AT::add(azr[j], zv[j] * rv[j]);
                    }
                    store_row<T, K>(r, p.row, rv);
                    store_row<T, K>(d, p.row, zv);
                }
            });
        team.sync();
    }
    team.template sum<T, K>(azr, zr);
}

// One iteration for the active columns. `update_d`: the backward sweep first forms
// d = z + beta d (not in a segment's first iteration, whose d = z the restart set).
template <typename T, int K, typename Team>
__device__ void eis_iterate(Team& team, const SellView& S, TeamControl<T, K>& ctl, const T* val, const T* wd,
                            const T* sd, T* r, T* d, T* m, T* q, T* c, bool update_d, double (&zr_new)[K]) {
    using AT = AccT<T>;
    using Acc = typename AT::type;
    const int n = S.n;
    const int lane = threadIdx.x & 31;
    const bool leader = threadIdx.x == 0;
    {   // backward sweep: technical = (d - U technical) w / D, with d = z + beta d first
        T beta[K];
        #pragma unroll
        for (int j = 0; j < K; j++) beta[j] = ctl.beta[j];
        for (int col = S.ncolors - 1; col >= 0; col--) {
            for_slices_dot<T, T, K, kBlockU>(team, S, __ldg(&S.color_slice[col]), __ldg(&S.color_slice[col + 1]),
                                             val, m,
                [&](const SliceMeta& M) {
                    RowState<T, K> p;
                    p.row = M.row0 + lane; p.act = lane < M.nrow;
                    p.w = p.act ? __ldg(&wd[p.row]) : T(0);
                    load_row<T, K>(d, p.row, p.act, p.a);
                    if (update_d) {
                        p.sdv = p.act ? __ldg(&sd[p.row]) : T(0);
                        load_row<T, K>(r, p.row, p.act, p.b);
                    }
                    return p;
                },
                [&](const SliceMeta&, const RowState<T, K>& p, const T (&sum)[K]) {
                    if (p.act && p.w != T(0)) {
                        T dv[K], mv[K];
                        #pragma unroll
                        for (int j = 0; j < K; j++) {
                            dv[j] = update_d ? p.b[j] * p.sdv + beta[j] * p.a[j] : p.a[j];
                            mv[j] = (dv[j] - sum[j]) * p.w;
                        }
                        if (update_d) store_row<T, K>(d, p.row, dv);
                        store_row<T, K>(m, p.row, mv);
                    }
                });
            team.sync();
        }
    }
    Acc dad[K];
    #pragma unroll
    for (int j = 0; j < K; j++) dad[j] = AT::zero();
    for (int col = 0; col < S.ncolors; col++) {              // forward sweep: auxiliary, d.(aux + tech)
        for_slices_dot<T, T, K, kBlockL>(team, S, __ldg(&S.color_slice[col]), __ldg(&S.color_slice[col + 1]), val, q,
            [&](const SliceMeta& M) {
                RowState<T, K> p;
                p.row = M.row0 + lane; p.act = lane < M.nrow;
                p.w = p.act ? __ldg(&wd[p.row]) : T(0);
                p.sdv = p.act ? __ldg(&sd[p.row]) : T(0);
                load_row<T, K>(d, p.row, p.act, p.a);
                load_row<T, K>(m, p.row, p.act, p.b);
                return p;
            },
            [&](const SliceMeta&, const RowState<T, K>& p, const T (&sum)[K]) {
                if (p.act && p.w != T(0)) {
                    T av[K];
                    #pragma unroll
                    for (int j = 0; j < K; j++) {
                        av[j] = (p.a[j] - p.sdv * p.b[j] - sum[j]) * p.w;
                        dad[j] = AT::add(dad[j], (av[j] + p.b[j]) * p.a[j]);
                    }
                    store_row<T, K>(q, p.row, av);
                }
            });
        team.sync();
    }
    {
        double dq[K];
        team.template sum<T, K>(dad, dq);
        if (leader) {
            int act = ctl.active;
            for (int j = 0; j < K; j++) {
                T a = T(0);
                if (act >> j & 1) {
                    const double zr = ctl.zr[j];
                    if (!(dq[j] > 0.0) || !(zr >= 0.0) || !isfinite(dq[j]) || !isfinite(zr)) act &= ~(1 << j);
                    else a = (T)(zr / dq[j]);
                }
                ctl.alpha[j] = a;
            }
            ctl.active = act;
        }
    }
    __syncthreads();
    Acc azr[K];
    {   // update: c += alpha technical, r -= alpha (auxiliary + technical), z.r with z = S r
        T alpha[K];
        #pragma unroll
        for (int j = 0; j < K; j++) { alpha[j] = ctl.alpha[j]; azr[j] = AT::zero(); }
        for (int i = team.tid(); i < n; i += team.nthreads()) {
            const T w = __ldg(&wd[i]);
            if (w == T(0)) continue;
            const T sdv = __ldg(&sd[i]);
            T cv[K], mv[K], qv[K], rv[K], zv[K];
            load_k_stream<T, K>(c + (long long)i * K, cv);
            load_k_stream<T, K>(m + (long long)i * K, mv);
            load_k_stream<T, K>(q + (long long)i * K, qv);
            load_k_stream<T, K>(r + (long long)i * K, rv);
            #pragma unroll
            for (int j = 0; j < K; j++) {
                cv[j] += alpha[j] * mv[j];
                rv[j] -= alpha[j] * (qv[j] + mv[j]);
                zv[j] = rv[j] * sdv;
                azr[j] = AT::add(azr[j], zv[j] * rv[j]);
            }
            store_row<T, K>(c, i, cv);
            store_row<T, K>(r, i, rv);
        }
    }
    team.template sum<T, K>(azr, zr_new);
}

// One team solves work item `it` completely.
template <typename T, int K, bool RAINBOW, typename Team>
__device__ void team_solve(Team& team, const BatchArgs& args, const BatchItem& it) {
    const SellView S = args.systems[it.system];
    const int n = S.n;
    const int lane = threadIdx.x & 31;
    const int kk = it.nrhs;                       // active columns (<= K)
    const T* val = sel_val<T>(S);
    const T* wd = sel_wd<T>(S);
    const T* sd = sel_sd<T>(S);
    double* xp = it.xp; double* bp = it.bp; double* r64 = it.r64;
    T* r = (T*)it.r; T* d = (T*)it.d; T* m = (T*)it.m; T* q = (T*)it.q; T* c = (T*)it.c;
    __shared__ TeamControl<T, K> ctl;
    const bool leader = threadIdx.x == 0;

    // gather caller vectors into the permuted, interleaved layout; ||b||^2
    for (int i = team.tid(); i < n; i += team.nthreads()) {
        const int o = __ldg(&S.perm[i]);
        #pragma unroll
        for (int j = 0; j < K; j++) {
            bp[(long long)i * K + j] = j < kk ? it.b[j][o] : 0.0;
            xp[(long long)i * K + j] = j < kk ? it.x[j][o] : 0.0;
        }
    }
    {
        double a2[K], o[K];
        #pragma unroll
        for (int j = 0; j < K; j++) a2[j] = 0.0;
        team.sync();
        for (int i = team.tid(); i < n; i += team.nthreads())
            #pragma unroll
            for (int j = 0; j < K; j++) { const double v = bp[(long long)i * K + j]; a2[j] += v * v; }
        team.template sum<double, K>(a2, o);
        if (leader) {
            ctl.done = 0;
            for (int j = 0; j < K; j++) {
                ctl.bnorm2[j] = o[j];
                ctl.iters[j] = 0; ctl.outer[j] = 0; ctl.status[j] = FEEC_MAXITER; ctl.relres[j] = -1.0;
                ctl.stall[j] = 0.0; ctl.amp[j] = 0.0; ctl.rnorm[j] = 0.0;
                ctl.beta[j] = T(0);
                if (j >= kk) ctl.done |= 1 << j;
            }
            ctl.err_step = 0; ctl.trig = 0;
        }
    }
    // Error control (mixed precision): a correction approximates the error of the iterate it
    // corrects, so its size against that iterate's residual measures the operator's
    // error-to-residual amplification; a column stops only when also max(amplification,
    // kAmpFloor) x relative residual <= kErrorPerResidual x precision, and each segment's
    // target is sized for both bars.
    const double err_target = kErrorPerResidual * args.precision;
    const double delta2 = args.inner_eta * args.inner_eta;   // segment factor, squared

    for (int seg = 0; ; seg++) {
        // ---- FP64 true residual r64 = b - A x and its norm ----
        team.sync();
        {
            double a2[K], rn2[K];
            #pragma unroll
            for (int j = 0; j < K; j++) a2[j] = 0.0;
            for_slices_dot<double, double, K, kBlockFull>(team, S, 0, S.nslices, S.val64, xp,
                [&](const SliceMeta& M) {
                    RowState<double, K> p;
                    p.row = M.row0 + lane; p.act = lane < M.nrow;
                    load_row<double, K>(bp, p.row, p.act, p.a);
                    return p;
                },
                [&](const SliceMeta&, const RowState<double, K>& p, const double (&sum)[K]) {
                    if (p.act) {
                        double rv[K];
                        #pragma unroll
                        for (int j = 0; j < K; j++) { rv[j] = p.a[j] - sum[j]; a2[j] += rv[j] * rv[j]; }
                        store_row<double, K>(r64, p.row, rv);
                    }
                });
            team.template sum<double, K>(a2, rn2);
            // stop tests and the scale of the next segment per column
            if (leader) {
                int done = ctl.done;
                for (int j = 0; j < kk; j++) {
                    const double bn = sqrt(ctl.bnorm2[j]);
                    const double rn = sqrt(rn2[j]);
                    const double rel = bn > 0.0 ? rn / bn : 0.0;
                    if (!(done >> j & 1)) {
                        int st = -1;
                        const bool budget = ctl.iters[j] >= args.max_iter || ctl.outer[j] >= args.max_outer;
                        if (!(rn == rn)) st = FEEC_BREAKDOWN;
                        else if (rn <= args.precision * bn) {
                            // stop at the error bar, or when the residual no longer falls (the FP64
                            // residual's own rounding floor) after the bar was first missed
                            const bool floor = (ctl.err_step >> j & 1) && rn > 0.3 * ctl.rnorm[j];
                            const double amp = ctl.amp[j] > kAmpFloor ? ctl.amp[j] : kAmpFloor;
                            if (!args.err_control || amp * rel <= err_target || budget || floor) st = FEEC_OK;
                            else ctl.err_step |= 1 << j;
                        } else if (args.stall_check && seg > 0 && (ctl.trig >> j & 1) && rn > ctl.stall[j]) {
                            st = kStatusStagnated;   // FP32 cannot follow: the host finishes it in FP64
                        } else if (budget) st = FEEC_MAXITER;
                        if (st >= 0) { done |= 1 << j; ctl.status[j] = st; }
                    }
                    ctl.relres[j] = rel;
                    const bool live = !(done >> j & 1);
                    ctl.inv[j] = live && rn > 0.0 ? (T)(1.0 / rn) : T(0);
                    ctl.rnorm[j] = live ? rn : 0.0;
                }
                for (int j = kk; j < K; j++) { ctl.inv[j] = T(0); ctl.rnorm[j] = 0.0; }
                ctl.trig = 0;
                ctl.done = done;
                ctl.all_done = done == (1 << K) - 1;
            }
        }
        __syncthreads();
        if (ctl.all_done) break;

        // ---- restart the inner iteration on the new residual ----
        {
            double zr[K];
            if constexpr (RAINBOW)
                eis_transform<T, K>(team, S, ctl, val, wd, sd, r64, r, d, m, q, c, seg == 0, zr);
            else
                cg_transform<T, K>(team, S, ctl, r64, r, d, c, zr);
            if (leader) {
                const int done = ctl.done;
                for (int j = 0; j < K; j++) {
                    const bool live = !(done >> j & 1);
                    ctl.beta[j] = T(0);
                    ctl.zr[j] = zr[j];
                    // the segment ends once z.r has fallen by delta^2 or far enough for the target
                    // (the residual bar and, once an amplification is known, the error bar),
                    // whichever comes first: the larger of the two factors
                    const double bn = sqrt(ctl.bnorm2[j]);
                    double target = args.precision * bn;
                    if (args.err_control) {
                        const double amp = ctl.amp[j] > kAmpFloor ? ctl.amp[j] : kAmpFloor;
                        if (err_target * bn / amp < target) target = err_target * bn / amp;
                    }
                    const double rn = ctl.rnorm[j];
                    const double need = rn > 0.0 ? args.inner_margin * target / rn : 0.0;
                    const double f = need * need > delta2 ? need * need : delta2;
                    ctl.thr[j] = live ? zr[j] * f : 0.0;
                    // the next true residual must gain at least half the digits z.r promised
                    ctl.stall[j] = rn * sqrt(sqrt(f > 0.0 ? f : 1.0));
                }
                ctl.active = ~done & ((1 << K) - 1);
            }
        }
        __syncthreads();

        // ---- iterate until a column's segment ends (the restart set d = z) ----
        bool update_d = false;
        while (true) {
            double zr_new[K];
            if constexpr (RAINBOW)
                eis_iterate<T, K>(team, S, ctl, val, wd, sd, r, d, m, q, c, update_d, zr_new);
            else
                cg_iterate<T, K>(team, S, ctl, val, r, d, q, c, zr_new);
            update_d = true;
            // a column whose z.r met its threshold (or whose budget ran out, or that broke
            // down) stops iterating; the segment ends when every column has stopped
            if (leader) {
                const int was = ctl.active;
                int act = was;
                for (int j = 0; j < K; j++) {
                    T b = T(0);
                    if (was >> j & 1) {
                        b = (T)(zr_new[j] / ctl.zr[j]);
                        ctl.zr[j] = zr_new[j];
                        ctl.iters[j]++;
                        if (!(zr_new[j] >= ctl.thr[j]) || ctl.iters[j] >= args.max_iter) act &= ~(1 << j);
                    }
                    if (!(act >> j & 1) && !(ctl.done >> j & 1)) ctl.trig |= 1 << j;
                    ctl.beta[j] = b;
                }
                ctl.active = act;
            }
            __syncthreads();
            if (!ctl.active) break;
            team.sync();
        }

        // ---- x += ||r64|| c in FP64, with the norms of the corrections and the new iterates ----
        {
            double rnorm[K], nn[2 * K], nsum[2 * K];
            #pragma unroll
            for (int j = 0; j < K; j++) { rnorm[j] = ctl.rnorm[j]; nn[j] = 0.0; nn[K + j] = 0.0; }
            const int done = ctl.done;
            for (int i = team.tid(); i < n; i += team.nthreads())
                #pragma unroll
                for (int j = 0; j < K; j++) {
                    const long long p = (long long)i * K + j;
                    if (!(done >> j & 1)) {
                        const double cj = rnorm[j] * (double)c[p];
                        const double xn = xp[p] + cj;
                        xp[p] = xn;
                        nn[j] += cj * cj;
                        nn[K + j] += xn * xn;
                    }
                }
            team.template sum<double, 2 * K>(nn, nsum);
            if (leader)
                for (int j = 0; j < K; j++) {
                    if (ctl.done >> j & 1) continue;
                    // the first segment starts from the initial guess (its correction is the
                    // solution); a later one measures the error of the iterate it corrected
                    if (ctl.outer[j] > 0 && nsum[K + j] > 0.0 && ctl.relres[j] > 0.0 && (ctl.trig >> j & 1)) {
                        const double a = sqrt(nsum[j] / nsum[K + j]) / ctl.relres[j];
                        if (a > ctl.amp[j]) ctl.amp[j] = a;
                    }
                    ctl.outer[j]++;
                }
        }
    }
    // scatter x back to the caller's numbering and report
    team.sync();
    for (int i = team.tid(); i < n; i += team.nthreads()) {
        const int o = __ldg(&S.perm[i]);
        #pragma unroll
        for (int j = 0; j < K; j++)
            if (j < kk) it.x[j][o] = xp[(long long)i * K + j];
    }
    if (team.rank() == 0 && leader) {
        for (int j = 0; j < kk; j++) {
            const int slot = it.first_result + j;
            args.results[slot].status = (ctl.done >> j & 1) ? ctl.status[j] : FEEC_MAXITER;
            args.results[slot].iterations = ctl.iters[j];
            args.results[slot].outer = ctl.outer[j];
            args.results[slot].relres = ctl.relres[j];
            // the bound the stop rule enforced: max(amplification, kAmpFloor) x relative residual
            const double amp = ctl.amp[j] > kAmpFloor ? ctl.amp[j] : kAmpFloor;
            args.results[slot].err_est = args.err_control ? amp * ctl.relres[j] : -1.0;
        }
    }
}

}  // namespace
}  // namespace team_solver
}  // namespace feec
