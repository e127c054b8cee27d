// Persistent Krylov solvers for sm_103a: one cooperative launch runs a whole
// solve. Every phase of the reference's iteration becomes a grid-stride sweep
// over rows, separated by bounded grid barriers; dot products are reduced
// deterministically (fixed shuffle tree per block, fixed-order sum of the
// per-block partials), so every block takes the same branch on the same bits.
//
//   cg_persistent  — ConjugateGradientSolverCSR   (solver/sparsesolver.cpp:26-201)
//   pcg_persistent — ConjugateGradientSolverCSR_SSOR (:446-724) and _Rainbow
//                    (:1002-1335): SSOR sweeps phase by phase over a schedule
//                    (colors for Rainbow, dependency levels for index-order SSOR)
//                    on a matrix whose rows are split into [L | E | U] parts.
//
// T = double is the drop-in FP64 path; T = float is the inner solver of the
// mixed-precision mode (FP32 storage, FP32 arithmetic, compensated FP32 dots).
#include <cmath>
#include <cstdio>
#include <type_traits>

#include "feec_device.cuh"
#include "feec_internal.h"
#include "persistent_common.cuh"

namespace feec {

// Pipelined row loops of the preconditioned solver. A group (LANES lanes) walks its
// row slots of a phase; the bounds of its next row and the first entries of that
// row's segment (column indices and values, PF per lane) are loaded while the
// current row is processed, and the first row of the next phase is loaded the same
// way before the grid barrier that separates the phases: the matrix is read-only,
// so only the gathered vector values have to wait for the barrier.
template <typename T, int LANES>
struct Prefetch {   // entries per lane, within the 64 registers of a thread
    static constexpr int value = sizeof(T) == 8 ? ((LANES >= 8) ? 1 : 2) : ((LANES >= 16) ? 1 : (LANES >= 8 ? 2 : 4));
};

template <typename T, int LANES>
struct RowRef {
    static constexpr int PF = Prefetch<T, LANES>::value;
    int i, a, e;        // row (-1: no row for this group), segment [a, e) of ci / val
    int c[PF];          // this lane's first PF entries: j = a + lane + t * LANES
    T v[PF];
};

enum { kRowsL = 0, kRowsBackwardU = 1, kRowsFull = 2 };

template <int KIND, int LANES, typename T>
__device__ __forceinline__ RowRef<T, LANES> row_ref(const PcgArgs<T>& a, int k, int hi) {
    RowRef<T, LANES> r;
    r.i = -1; r.a = 0; r.e = 0;
    if (k < hi) {
        if (KIND == kRowsBackwardU) {
            r.i = __ldg(&a.brows[k]);
            r.a = __ldg(&a.usplit[r.i]);
            r.e = __ldg(&a.rp[r.i + 1]);
        } else {
            r.i = k;
            r.a = __ldg(&a.rp[k]);
            r.e = (KIND == kRowsL) ? __ldg(&a.lsplit[k]) : __ldg(&a.rp[k + 1]);
        }
    }
    const int lane = threadIdx.x & (LANES - 1);
    #pragma unroll
    for (int t = 0; t < RowRef<T, LANES>::PF; t++) {
        const int j = r.a + lane + t * LANES;
        const bool ok = j < r.e;
        r.c[t] = ok ? __ldg(&a.ci[j]) : 0;
        r.v[t] = ok ? __ldg(&a.val[j]) : T(0);
    }
    return r;
}

// seg_dot over a prefetched row: the same terms in the same order as seg_dot.
template <typename T, int LANES>
__device__ __forceinline__ T seg_dot_pre(const RowRef<T, LANES>& R, const int* __restrict__ ci,
                                         const T* __restrict__ v, const T* x, int lane) {
    constexpr int PF = RowRef<T, LANES>::PF;
    T s = T(0);
    #pragma unroll
    for (int t = 0; t < PF; t++)
        if (R.a + lane + t * LANES < R.e) s = fma(R.v[t], x[R.c[t]], s);
    s = seg_accumulate<T, LANES>(ci, v, x, R.a + lane + PF * LANES, R.e, s);
    #pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off, LANES);
    return s;
}

template <int LANES>
__device__ __forceinline__ int group_base(int lo) {
    return lo + (int)((blockIdx.x * blockDim.x + threadIdx.x) / 32) * (32 / LANES);
}
template <int LANES>
__device__ __forceinline__ int group_first(int lo) {
    return group_base<LANES>(lo) + (int)((threadIdx.x & 31) / LANES);
}
template <int LANES>
__device__ __forceinline__ int group_stride() {
    return (int)(gridDim.x * blockDim.x / 32) * (32 / LANES);
}

template <int LANES, int KIND, typename T, typename F>
__device__ __forceinline__ void rows_pipelined(const PcgArgs<T>& a, int lo, int hi, RowRef<T, LANES> cur, F&& body) {
    const int stride = group_stride<LANES>();
    int k = group_first<LANES>(lo);
    for (int base = group_base<LANES>(lo); base < hi; base += stride, k += stride) {
        const RowRef<T, LANES> nxt = row_ref<KIND, LANES>(a, k + stride, hi);
        body(cur);
        cur = nxt;
    }
}

// ---------------------------------------------------------------------------
// Plain CG
// ---------------------------------------------------------------------------
template <typename T, int LANES>
__global__ void __launch_bounds__(kThreads, 2) cg_persistent(CgArgs<T> a) {
    using AT = AccT<T>;
    using Acc = typename AT::type;
    unsigned long long epoch = 0;
    const int n = a.n;
    const int lane = threadIdx.x & (LANES - 1);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nthr = gridDim.x * blockDim.x;
    double* p_dq = a.partials;
    double* p_rr = a.partials + gridDim.x;

    // With a diagonal preconditioner (sparsesolver.cpp:221-416) z = precon r replaces r in
    // the direction and the scalar products, and rows with precon == 0 are skipped.
    const T* pc = a.precon;
    // restart (sparsesolver.cpp:76-104 / :283-302): r = b - A x, d = r (or z), r.r (or z.r)
    Acc acc = AT::zero();
    FEEC_FOR_ROW_GROUPS(0, n, i, act) {
        const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
        const T s = seg_dot<T, LANES>(a.ci, a.val, a.x, lo, hi, lane);
        if (act && lane == 0) {
            if (pc) {
                const T p = __ldg(&pc[i]);
                if (p != T(0)) {
                    const T ri = __ldg(&a.b[i]) - s;
                    a.r[i] = ri;
                    const T zi = p * ri;
                    a.z[i] = zi;
                    a.d[i] = zi;
                    acc = AT::add(acc, zi * ri);
                }
            } else {
                const T ri = __ldg(&a.b[i]) - s;
                a.r[i] = ri;
                if (!a.keep_dir) a.d[i] = ri;
                acc = AT::add(acc, ri * ri);
            }
        }
    }
    write_partials<T>(p_rr, acc);
    if (!grid_barrier(a.st, epoch, 1)) return;
    double rr[1];
    grid_sum<1>(p_rr, rr);
    double r_r = rr[0];
    double r_r_prev = r_r;
    if (a.keep_dir && !pc) {
        // reliable update: the previous segment's direction continues the recurrence,
        // d = r + beta d with beta against its rho, rescaled to the new residual scale
        const T beta0 = (T)(r_r / (a.zr_prev * a.scale));
        for (int i = tid; i < n; i += nthr) a.d[i] = a.r[i] + beta0 * a.d[i];
        if (!grid_barrier(a.st, epoch, 5)) return;
    }

    // Scalar control (stop tests, alpha, beta) is evaluated by thread 0 only and
    // broadcast through shared memory: FP64 issues at 2 lanes/clk/SM on this part,
    // so redundant per-thread FP64 scalar work would cost more than the sweeps.
    __shared__ double s_scal[2];
    __shared__ int s_ctl;
    int K = 0;
    int status = FEEC_MAXITER;
    double d_Ad = 0.0;
    while (K < a.max_iter) {
        if (threadIdx.x == 0) {
            if (a.print_modulo > 0 && K % a.print_modulo == 0 && blockIdx.x == 0)
                printf("(%d/%d)   INTERIM: Residual norm is %.9le < %.9le\n", K, n, sqrt(r_r), a.print_tol);
            s_ctl = fabs(r_r) < a.tol2 ? 1 : 0;                                          // :116-119
        }
        __syncthreads();
        if (s_ctl) { status = FEEC_OK; break; }

        // q = A d, d.q                                                               :126-139
        Acc adq = AT::zero();
        FEEC_FOR_ROW_GROUPS(0, n, i, act) {
            const bool live = act && (!pc || __ldg(&pc[i]) != T(0));
            const int lo = live ? __ldg(&a.rp[i]) : 0, hi = live ? __ldg(&a.rp[i + 1]) : 0;
            const T s = seg_dot<T, LANES>(a.ci, a.val, a.d, lo, hi, lane);
            if (live && lane == 0) {
                a.q[i] = s;
                adq = AT::add(adq, a.d[i] * s);
            }
        }
        write_partials<T>(p_dq, adq);
        if (!grid_barrier(a.st, epoch, 2)) return;
        double dq[1];
        grid_sum<1>(p_dq, dq);
        d_Ad = dq[0];
        if (threadIdx.x == 0) {
            int ctl = 0;
            if (!isfinite(r_r) || r_r < 0.0 || !isfinite(d_Ad) || d_Ad < 0.0) ctl = 1;   // :142-151
            else if (sqrt(fabs(d_Ad)) < kMachineEpsilon) ctl = 2;                         // :153-157
            s_ctl = ctl;
            s_scal[0] = r_r / d_Ad;
        }
        __syncthreads();
        if (s_ctl == 1) { status = FEEC_BREAKDOWN; break; }
        if (s_ctl == 2) { status = FEEC_SMALL_ENERGY; break; }

        const T alpha = (T)s_scal[0];
        Acc arr = AT::zero();
        for (int i = tid; i < n; i += nthr) {                                          // :158-173 / :361-378
            T p = T(1);
            if (pc) { p = __ldg(&pc[i]); if (p == T(0)) continue; }
            const T di = a.d[i];
            a.x[i] += alpha * di;
            const T ri = a.r[i] - alpha * a.q[i];
            a.r[i] = ri;
            if (pc) {
                const T zi = p * ri;
                a.z[i] = zi;
                arr = AT::add(arr, zi * ri);
            } else {
                arr = AT::add(arr, ri * ri);
            }
        }
        write_partials<T>(p_rr, arr);
        if (!grid_barrier(a.st, epoch, 3)) return;
        grid_sum<1>(p_rr, rr);
        const double r_r_new = rr[0];
        if (threadIdx.x == 0) s_scal[1] = r_r_new / r_r;                               // :175-183
        __syncthreads();
        const T beta = (T)s_scal[1];
        r_r_prev = r_r;
        r_r = r_r_new;
        if (pc) {
            for (int i = tid; i < n; i += nthr)
                if (__ldg(&pc[i]) != T(0)) a.d[i] = a.z[i] + beta * a.d[i];            // :386-395
        } else {
            for (int i = tid; i < n; i += nthr) a.d[i] = a.r[i] + beta * a.d[i];
        }
        if (!grid_barrier(a.st, epoch, 4)) return;
        K++;
    }
    finish(a.st, status, K, r_r, d_Ad);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st->extra[0] = r_r_prev;
}

// ---------------------------------------------------------------------------
// SSOR / multicolor SSOR preconditioned CG
// ---------------------------------------------------------------------------
// Two co-resident 512-thread blocks per SM (64 registers per thread): the phases are
// latency-bound, so warps in flight matter more than registers.
template <typename T, int LANES>
__global__ void __launch_bounds__(kThreads, 2) pcg_persistent(PcgArgs<T> a) {
    using AT = AccT<T>;
    using Acc = typename AT::type;
    unsigned long long epoch = 0;
    const int n = a.n;
    const int lane = threadIdx.x & (LANES - 1);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nthr = gridDim.x * blockDim.x;
    double* p_dq = a.partials;
    double* p_zr = a.partials + gridDim.x;   // (z.r, r.r) pairs
    // Per-row factors prepared at setup: wd = omega / D (0 where D == 0, the rows the
    // reference skips), sd = D (2 - omega) / omega. The sweeps then need no division.
    __shared__ double s_scal[2];
    __shared__ int s_ctl;

    // ---- restart (sparsesolver.cpp:1072-1175 / 506-588) ----
    Acc arr = AT::zero();
    FEEC_FOR_ROW_GROUPS(0, n, i, act) {                      // r = b - A x for rows with D != 0
        const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
        const T s = seg_dot<T, LANES>(a.ci, a.val, a.x, lo, hi, lane);
        if (act && lane == 0 && __ldg(&a.wd[i]) != T(0)) {
            const T ri = __ldg(&a.b[i]) - s;
            a.r[i] = ri;
            arr = AT::add(arr, ri * ri);
        }
    }
    if (!grid_barrier(a.st, epoch, 10)) return;
    for (int p = 0; p < a.nf; p++) {                          // forward sweep, phase by phase
        const int lo_r = __ldg(&a.fptr[p]), hi_r = __ldg(&a.fptr[p + 1]);
        FEEC_FOR_ROW_GROUPS(lo_r, hi_r, i, act) {
            const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.lsplit[i]) : 0;
            const T s = seg_dot<T, LANES>(a.ci, a.val, a.m, lo, hi, lane);
            if (act && lane == 0) {
                const T w = __ldg(&a.wd[i]);
                if (w != T(0)) a.m[i] = (a.r[i] - s) * w;
            }
        }
        if (!grid_barrier(a.st, epoch, 11)) return;
    }
    Acc azr = AT::zero();
    for (int p = 0; p < a.nbw; p++) {                         // scale + backward sweep
        const int lo_r = __ldg(&a.bptr[p]), hi_r = __ldg(&a.bptr[p + 1]);
        FEEC_FOR_ROW_GROUPS(lo_r, hi_r, k, act) {
            const int i = act ? __ldg(&a.brows[k]) : 0;
            const int lo = act ? __ldg(&a.usplit[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
            const T s = seg_dot<T, LANES>(a.ci, a.val, a.z, lo, hi, lane);
            if (act && lane == 0) {
                const T w = __ldg(&a.wd[i]);
                if (w != T(0)) {
                    const T mi = a.m[i] * __ldg(&a.sd[i]);
                    a.m[i] = mi;
                    const T zi = (mi - s) * w;
                    a.z[i] = zi;
                    a.d[i] = zi;
                    azr = AT::add(azr, zi * a.r[i]);
                }
            }
        }
        if (p + 1 < a.nbw) {
            if (!grid_barrier(a.st, epoch, 12)) return;
        }
    }
    write_partials2<T>(p_zr, azr, arr);
    if (!grid_barrier(a.st, epoch, 13)) return;
    double zr2[2];
    grid_sum<2>(p_zr, zr2);
    double z_r = zr2[0], r_r = zr2[1];

    int K = 0;
    int status = FEEC_MAXITER;
    double d_Ad = 0.0;
    RowRef<T, LANES> pf = row_ref<kRowsFull, LANES>(a, group_first<LANES>(0), n);
    constexpr int LL = LANES > kLongLanes ? LANES : kLongLanes;   // long rows of multicolor phases
    while (K < a.max_iter) {
        if (threadIdx.x == 0) {
            if (a.print_modulo > 0 && K % a.print_modulo == 0 && blockIdx.x == 0)
                printf("(%d/%d)   INTERIM: Residual norm is %.9le < %.9le\n", K, n, sqrt(z_r), a.print_tol);
            int ctl = 0;
            if (a.use_zr_rule && fabs(z_r) < a.tol2) ctl = 1;                         // :1187-1190
            if (a.rr_stop > 0.0 && r_r < a.rr_stop) ctl = 1;
            s_ctl = ctl;
        }
        __syncthreads();
        if (s_ctl) { status = FEEC_OK; break; }

        Acc adq = AT::zero();                                                          // :1197-1212
        rows_pipelined<LANES, kRowsFull>(a, 0, n, pf, [&](const RowRef<T, LANES>& R) {
            const bool act = R.i >= 0;
            const T s = seg_dot_pre<T, LANES>(R, a.ci, a.val, a.d, lane);
            if (act && lane == 0) {
                const T qi = (__ldg(&a.wd[R.i]) != T(0)) ? s : T(0);
                a.q[R.i] = qi;
                adq = AT::add(adq, a.d[R.i] * qi);
            }
        });
        write_partials<T>(p_dq, adq);
        int flo = __ldg(&a.fptr[0]), fhi = __ldg(&a.fptr[1]);
        pf = row_ref<kRowsL, LANES>(a, group_first<LANES>(flo), fhi);
        if (!grid_barrier(a.st, epoch, 14)) return;
        double dq[1];
        grid_sum<1>(p_dq, dq);
        d_Ad = dq[0];
        if (threadIdx.x == 0) {
            int ctl = 0;
            if (!isfinite(z_r) || z_r < 0.0 || !isfinite(d_Ad) || d_Ad < 0.0) ctl = 1;
            else if (sqrt(fabs(d_Ad)) < kMachineEpsilon) ctl = 2;
            s_ctl = ctl;
            s_scal[0] = z_r / d_Ad;
        }
        __syncthreads();
        if (s_ctl == 1) { status = FEEC_BREAKDOWN; break; }
        if (s_ctl == 2) { status = FEEC_SMALL_ENERGY; break; }

        const T alpha = (T)s_scal[0];
        arr = AT::zero();
        if (a.fsplit) {
            // multicolor phases with long rows first: split lane counts (split_rows)
            for (int p = 0; p < a.nf; p++) {                                           // :1230-1261
                const int lo_r = __ldg(&a.fptr[p]), sp_r = __ldg(&a.fsplit[p]), hi_r = __ldg(&a.fptr[p + 1]);
                split_rows<LANES, LL>(lo_r, sp_r, hi_r, [&](auto L, int i, bool act, int ln) {
                    constexpr int LN = decltype(L)::value;
                    const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.lsplit[i]) : 0;
                    // the row's own values are requested before its entries' gathers
                    T w = T(0), xi = T(0), di = T(0), ri0 = T(0), qi = T(0);
                    if (act && ln == 0) { w = __ldg(&a.wd[i]); xi = a.x[i]; di = a.d[i]; ri0 = a.r[i]; qi = a.q[i]; }
                    const T s = seg_dot<T, LN>(a.ci, a.val, a.m, lo, hi, ln);
                    if (act && ln == 0 && w != T(0)) {
                        a.x[i] = xi + alpha * di;
                        const T ri = ri0 - alpha * qi;
                        a.r[i] = ri;
                        arr = AT::add(arr, ri * ri);
                        a.m[i] = (ri - s) * w;
                    }
                });
                if (!grid_barrier(a.st, epoch, 15)) return;
            }
            azr = AT::zero();
            for (int p = 0; p < a.nbw; p++) {                                          // :1263-1307
                const int lo_r = __ldg(&a.bptr[p]), sp_r = __ldg(&a.bsplit[p]), hi_r = __ldg(&a.bptr[p + 1]);
                split_rows<LANES, LL>(lo_r, sp_r, hi_r, [&](auto L, int k, bool act, int ln) {
                    constexpr int LN = decltype(L)::value;
                    const int i = act ? __ldg(&a.brows[k]) : 0;
                    const int lo = act ? __ldg(&a.usplit[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
                    T w = T(0), m0 = T(0), sdi = T(0), ri = T(0);
                    if (act && ln == 0) { w = __ldg(&a.wd[i]); m0 = a.m[i]; sdi = __ldg(&a.sd[i]); ri = a.r[i]; }
                    const T s = seg_dot<T, LN>(a.ci, a.val, a.z, lo, hi, ln);
                    if (act && ln == 0 && w != T(0)) {
                        const T mi = m0 * sdi;
                        a.m[i] = mi;
                        const T zi = (mi - s) * w;
                        a.z[i] = zi;
                        azr = AT::add(azr, zi * ri);
                    }
                });
                if (p + 1 < a.nbw && !grid_barrier(a.st, epoch, 16)) return;
            }
        } else {
        for (int p = 0; p < a.nf; p++) {                                               // :1230-1261
            rows_pipelined<LANES, kRowsL>(a, flo, fhi, pf, [&](const RowRef<T, LANES>& R) {
                const bool act = R.i >= 0;
                const T s = seg_dot_pre<T, LANES>(R, a.ci, a.val, a.m, lane);
                if (act && lane == 0) {
                    const T w = __ldg(&a.wd[R.i]);
                    if (w != T(0)) {
                        a.x[R.i] += alpha * a.d[R.i];
                        const T ri = a.r[R.i] - alpha * a.q[R.i];
                        a.r[R.i] = ri;
                        arr = AT::add(arr, ri * ri);
                        a.m[R.i] = (ri - s) * w;
                    }
                }
            });
            if (p + 1 < a.nf) {
                flo = fhi;
                fhi = __ldg(&a.fptr[p + 2]);
                pf = row_ref<kRowsL, LANES>(a, group_first<LANES>(flo), fhi);
            } else {
                pf = row_ref<kRowsBackwardU, LANES>(a, group_first<LANES>(__ldg(&a.bptr[0])), __ldg(&a.bptr[1]));
            }
            if (!grid_barrier(a.st, epoch, 15)) return;
        }
        azr = AT::zero();
        for (int p = 0; p < a.nbw; p++) {                                              // :1263-1307
            const int lo_r = __ldg(&a.bptr[p]), hi_r = __ldg(&a.bptr[p + 1]);
            rows_pipelined<LANES, kRowsBackwardU>(a, lo_r, hi_r, pf, [&](const RowRef<T, LANES>& R) {
                const bool act = R.i >= 0;
                const T s = seg_dot_pre<T, LANES>(R, a.ci, a.val, a.z, lane);
                if (act && lane == 0) {
                    const T w = __ldg(&a.wd[R.i]);
                    if (w != T(0)) {
                        const T mi = a.m[R.i] * __ldg(&a.sd[R.i]);
                        a.m[R.i] = mi;
                        const T zi = (mi - s) * w;
                        a.z[R.i] = zi;
                        azr = AT::add(azr, zi * a.r[R.i]);
                    }
                }
            });
            if (p + 1 < a.nbw) {
                pf = row_ref<kRowsBackwardU, LANES>(a, group_first<LANES>(hi_r), __ldg(&a.bptr[p + 2]));
                if (!grid_barrier(a.st, epoch, 16)) return;
            }
        }
        }
        pf = row_ref<kRowsFull, LANES>(a, group_first<LANES>(0), n);
        write_partials2<T>(p_zr, azr, arr);
        if (!grid_barrier(a.st, epoch, 17)) return;
        grid_sum<2>(p_zr, zr2);
        const double z_r_new = zr2[0];
        r_r = zr2[1];
        if (threadIdx.x == 0) s_scal[1] = z_r_new / z_r;                               // :1309-1318
        __syncthreads();
        const T beta = (T)s_scal[1];
        z_r = z_r_new;
        for (int i = tid; i < n; i += nthr) {
            if (__ldg(&a.wd[i]) != T(0)) a.d[i] = a.z[i] + beta * a.d[i];
        }
        if (!grid_barrier(a.st, epoch, 18)) return;
        K++;
    }
    finish(a.st, status, K, z_r, r_r);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
template <typename T, int LANES>
static const void* cg_fn() { return (const void*)cg_persistent<T, LANES>; }
template <typename T, int LANES>
static const void* pcg_fn() { return (const void*)pcg_persistent<T, LANES>; }

template <typename T>
static const void* family_fn(int family, int lanes) {
    if (family == 0) {
        switch (lanes) {
            case 1: return cg_fn<T, 1>(); case 2: return cg_fn<T, 2>(); case 4: return cg_fn<T, 4>();
            case 8: return cg_fn<T, 8>(); case 16: return cg_fn<T, 16>(); default: return cg_fn<T, 32>();
        }
    }
    switch (lanes) {
        case 1: return pcg_fn<T, 1>(); case 2: return pcg_fn<T, 2>(); case 4: return pcg_fn<T, 4>();
        case 8: return pcg_fn<T, 8>(); case 16: return pcg_fn<T, 16>(); default: return pcg_fn<T, 32>();
    }
}

int max_coresident_blocks(int family, int is_float, int lanes, int threads) {
    const void* fn = is_float ? family_fn<float>(family, lanes) : family_fn<double>(family, lanes);
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess) return 0;
    return sms * per_sm;
}

int pick_lanes(double avg) {
    if (avg <= 3.0) return 2;
    if (avg <= 10.0) return 4;
    if (avg <= 24.0) return 8;
    if (avg <= 48.0) return 16;
    return 32;
}

static int pick_blocks(int family, int is_float, int n, LaunchShape& shape) {
    if (shape.threads <= 0) shape.threads = kThreads;
    const int maxb = max_coresident_blocks(family, is_float, shape.lanes, shape.threads);
    if (maxb <= 0) return 0;
    // enough groups for every row in one sweep, at most the co-resident grid
    const long long want = ((long long)n * shape.lanes + shape.threads - 1) / shape.threads;
    int b = shape.blocks > 0 ? shape.blocks : (int)(want < maxb ? want : maxb);
    if (b > maxb) b = maxb;
    if (b < 1) b = 1;
    shape.blocks = b;
    return b;
}

template <typename T>
cudaError_t launch_cg(const CgArgs<T>& a, LaunchShape& shape, cudaStream_t s) {
    const int is_float = sizeof(T) == 4;
    if (pick_blocks(0, is_float, a.n, shape) <= 0) return cudaErrorInvalidConfiguration;
    CgArgs<T> copy = a;
    void* args[] = {&copy};
    note_launch();
    return cudaLaunchCooperativeKernel(family_fn<T>(0, shape.lanes), dim3(shape.blocks), dim3(shape.threads), args, 0, s);
}

template <typename T>
cudaError_t launch_pcg(const PcgArgs<T>& a, LaunchShape& shape, cudaStream_t s) {
    const int is_float = sizeof(T) == 4;
    if (pick_blocks(1, is_float, a.n, shape) <= 0) return cudaErrorInvalidConfiguration;
    PcgArgs<T> copy = a;
    void* args[] = {&copy};
    note_launch();
    return cudaLaunchCooperativeKernel(family_fn<T>(1, shape.lanes), dim3(shape.blocks), dim3(shape.threads), args, 0, s);
}

template cudaError_t launch_cg<double>(const CgArgs<double>&, LaunchShape&, cudaStream_t);
template cudaError_t launch_cg<float>(const CgArgs<float>&, LaunchShape&, cudaStream_t);
template cudaError_t launch_pcg<double>(const PcgArgs<double>&, LaunchShape&, cudaStream_t);
template cudaError_t launch_pcg<float>(const PcgArgs<float>&, LaunchShape&, cudaStream_t);

}  // namespace feec
