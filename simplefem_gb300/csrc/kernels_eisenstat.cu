// SSOR-PCG with Eisenstat's trick as one persistent cooperative launch:
//
//   ConjugateGradientSolverCSR_SSOR_Eisenstat   (solver/sparsesolver.cpp:726-995)
//   ConjugateGradientSolverCSR_Eisenstat_Rainbow (solver/sparsesolver.cpp:1338-1645)
//
// CG runs on the split-preconditioned system, so an iteration needs no SpMV: one
// backward sweep (technical = (D/w + U)^-1 direction), one forward sweep
// (auxiliary = (D/w + L)^-1 (direction - (2/w - 1) D technical)), and the update
// with auxiliary + technical playing the role of A direction. The sweeps run phase
// by phase over the same schedules as the SSOR / Rainbow solvers (dependency levels
// or colors) on rows split [L | E | U]; grid barriers separate dependent phases.
//
// Fusions that keep every per-row operation of the reference: the direction update
// d = z + beta d of the previous iteration runs in the backward sweep (a row's
// direction is only ever read by its own row), and auxiliary + technical and the
// direction . (auxiliary + technical) sum run in the forward sweep, into a separate
// vector because later colors still gather the pure auxiliary. An iteration has
// 2 * phases + 2 grid barriers. T = double is the drop-in (the reference's stopping rule);
// T = float is the inner solve of the mixed-precision mode (stops when z.r has fallen by
// a given factor, compensated FP32 sums).
#include <cmath>
#include <cstdio>

#include "feec_device.cuh"
#include "feec_internal.h"
#include "persistent_common.cuh"

namespace feec {
namespace {

// seg_dot that can skip entries whose column has D == 0 (the reference's
// `diagonal[csrcolumns[d]] != 0.` guard; wd = omega / D is 0 exactly there).
template <typename T, int LANES>
__device__ __forceinline__ T seg_dot_guarded(const int* __restrict__ ci, const T* __restrict__ v, const T* x,
                                             const T* __restrict__ wd, int lo, int hi, int lane, bool guard) {
    T s = T(0);
    if (guard) {
        for (int j = lo + lane; j < hi; j += LANES) {
            const int c = __ldg(&ci[j]);
            if (__ldg(&wd[c]) != T(0)) s = fma(__ldg(&v[j]), x[c], s);
        }
    } else {
        s = seg_accumulate<T, LANES>(ci, v, x, lo + lane, hi, s);
    }
    #pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off, LANES);
    return s;
}

// Vectors: r = residual (of the L-solved system, as the reference keeps it),
// d = direction, z = zirconium, m = technical, q = auxiliary, w = auxiliary + technical.
template <typename T, int LANES>
__global__ void __launch_bounds__(kThreads, 2) eisenstat_persistent(PcgArgs<T> a) {
    using AT = AccT<T>;
    using Acc = typename AT::type;
    unsigned long long epoch = 0;
    const int n = a.n;
    const int lane = threadIdx.x & (LANES - 1);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nthr = gridDim.x * blockDim.x;
    const bool g_restart = a.guard_restart != 0, g_iter = a.guard_iter != 0;
    const T c2 = (T)(2.0 / a.omega - 1.0);
    // two partial-sum arrays, used alternately: a block writes one only after a grid
    // barrier has passed since every block last read it
    double* p_dad = a.partials;
    double* p_zr = a.partials + gridDim.x;
    __shared__ double s_scal[2];
    __shared__ int s_ctl;

    // ---- restart (:786-842 / :1409-1478): auxiliary = b - A x, forward solve into r ----
    FEEC_FOR_ROW_GROUPS(0, n, i, act) {
        const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
        const T s = seg_dot_guarded<T, LANES>(a.ci, a.val, a.x, a.wd, lo, hi, lane, g_restart);
        if (act && lane == 0 && __ldg(&a.wd[i]) != T(0)) a.q[i] = __ldg(&a.b[i]) - s;
    }
    if (!grid_barrier(a.st, epoch, 30)) return;
    for (int p = 0; p < a.nf; p++) {
        const int lo_r = __ldg(&a.fptr[p]), hi_r = __ldg(&a.fptr[p + 1]);
        FEEC_FOR_ROW_GROUPS(lo_r, hi_r, i, act) {
            const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.lsplit[i]) : 0;
            const T s = seg_dot_guarded<T, LANES>(a.ci, a.val, a.r, a.wd, lo, hi, lane, g_restart);
            if (act && lane == 0) {
                const T w = __ldg(&a.wd[i]);
                if (w != T(0)) a.r[i] = (a.q[i] - s) * w;
            }
        }
        if (!grid_barrier(a.st, epoch, 31)) return;
    }
    const bool keep = a.keep_dir != 0;
    constexpr int LL = LANES > kLongLanes ? LANES : kLongLanes;   // long rows of multicolor phases
    Acc azr = AT::zero();
    for (int i = tid; i < n; i += nthr) {
        if (__ldg(&a.wd[i]) == T(0)) continue;
        const T ri = a.r[i];
        const T zi = ri * __ldg(&a.sd[i]);
        a.z[i] = zi;
        if (!keep) a.d[i] = zi;
        azr = AT::add(azr, zi * ri);
    }
    write_partials<T>(p_zr, azr);
    if (!grid_barrier(a.st, epoch, 32)) return;
    double one[1];
    grid_sum<1>(p_zr, one);
    double z_r = one[0];
    const double z_r0 = z_r;
    double z_r_prev = z_r;

    int K = 0;
    int status = FEEC_MAXITER;
    // a kept direction (reliable update) continues the recurrence: the first backward sweep
    // forms d = z + beta d with beta against the previous segment's rho, rescaled
    T beta = keep ? (T)(z_r / (a.zr_prev * a.scale)) : T(0);
    while (K < a.max_iter) {
        if (threadIdx.x == 0) {
            if (a.print_modulo > 0 && K % a.print_modulo == 0 && blockIdx.x == 0)
                printf("(%d/%d)   INTERIM: Residual norm is %.9le < %.9le\n", K, n, sqrt(z_r), a.print_tol);
            int ctl = (a.use_zr_rule && fabs(z_r) < a.tol2) ? 1 : 0;                     // :859-862
            if (a.rr_stop > 0.0 && z_r < a.rr_stop * z_r0) ctl = 1;                       // relative (inner solves)
            s_ctl = ctl;
        }
        __syncthreads();
        if (s_ctl) { status = FEEC_OK; break; }

        // backward sweep (:870-884 / :1506-1530), with the previous iteration's d = z + beta d;
        // in multicolor layouts each color's long rows get LL lanes (split_rows)
        for (int p = 0; p < a.nbw; p++) {
            const int lo_r = __ldg(&a.bptr[p]), hi_r = __ldg(&a.bptr[p + 1]);
            auto brow = [&](auto L, int k, bool act, int ln) {
                constexpr int LN = decltype(L)::value;
                const int i = act ? __ldg(&a.brows[k]) : 0;
                const int lo = act ? __ldg(&a.usplit[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
                const T s = seg_dot_guarded<T, LN>(a.ci, a.val, a.m, a.wd, lo, hi, ln, g_iter);
                if (act && ln == 0) {
                    const T w = __ldg(&a.wd[i]);
                    if (w != T(0)) {
                        T dv = a.d[i];
                        if (K > 0 || keep) { dv = a.z[i] + beta * dv; a.d[i] = dv; }        // :990-997
                        a.m[i] = (dv - s) * w;
                    }
                }
            };
            if (a.bsplit) {
                split_rows<LANES, LL>(lo_r, __ldg(&a.bsplit[p]), hi_r, brow);
            } else {
                FEEC_FOR_ROW_GROUPS(lo_r, hi_r, k, act) brow(std::integral_constant<int, LANES>{}, k, act, lane);
            }
            if (!grid_barrier(a.st, epoch, 33)) return;
        }
        // forward sweep (:886-914 / :1533-1571) with auxiliary + technical and d . (auxiliary + technical)
        Acc dad = AT::zero();
        for (int p = 0; p < a.nf; p++) {
            const int lo_r = __ldg(&a.fptr[p]), hi_r = __ldg(&a.fptr[p + 1]);
            auto frow = [&](auto L, int i, bool act, int ln) {
                constexpr int LN = decltype(L)::value;
                const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.lsplit[i]) : 0;
                const T s = seg_dot_guarded<T, LN>(a.ci, a.val, a.q, a.wd, lo, hi, ln, g_iter);
                if (act && ln == 0) {
                    const T w = __ldg(&a.wd[i]);
                    if (w != T(0)) {
                        const T dv = a.d[i], tv = a.m[i];
                        const T av = (dv - c2 * __ldg(&a.dg[i]) * tv - s) * w;
                        a.q[i] = av;
                        const T cv = av + tv;
                        a.w[i] = cv;
                        dad = AT::add(dad, cv * dv);
                    }
                }
            };
            if (a.fsplit) {
                split_rows<LANES, LL>(lo_r, __ldg(&a.fsplit[p]), hi_r, frow);
            } else {
                FEEC_FOR_ROW_GROUPS(lo_r, hi_r, i, act) frow(std::integral_constant<int, LANES>{}, i, act, lane);
            }
            if (p + 1 < a.nf && !grid_barrier(a.st, epoch, 34)) return;
        }
        write_partials<T>(p_dad, dad);
        if (!grid_barrier(a.st, epoch, 35)) return;
        grid_sum<1>(p_dad, one);
        const double d_Ad = one[0];
        if (threadIdx.x == 0) {                                                           // :918-933
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

        // update (:936-975): x += alpha technical, r -= alpha (auxiliary + technical), z, z.r
        Acc zrn = AT::zero();
        for (int i = tid; i < n; i += nthr) {
            if (__ldg(&a.wd[i]) == T(0)) continue;
            a.x[i] += alpha * a.m[i];
            const T ri = a.r[i] - alpha * a.w[i];
            a.r[i] = ri;
            const T zi = ri * __ldg(&a.sd[i]);
            a.z[i] = zi;
            zrn = AT::add(zrn, zi * ri);
        }
        write_partials<T>(p_zr, zrn);
        if (!grid_barrier(a.st, epoch, 36)) return;
        grid_sum<1>(p_zr, one);
        if (threadIdx.x == 0) s_scal[1] = one[0] / z_r;
        __syncthreads();
        beta = (T)s_scal[1];
        z_r_prev = z_r;
        z_r = one[0];
        K++;
    }
    finish(a.st, status, K, z_r, 0.0);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st->extra[0] = z_r_prev;
}

template <typename T>
const void* eisenstat_fn(int lanes) {
    switch (lanes) {
        case 1: return (const void*)eisenstat_persistent<T, 1>;
        case 2: return (const void*)eisenstat_persistent<T, 2>;
        case 4: return (const void*)eisenstat_persistent<T, 4>;
        case 8: return (const void*)eisenstat_persistent<T, 8>;
        case 16: return (const void*)eisenstat_persistent<T, 16>;
        default: return (const void*)eisenstat_persistent<T, 32>;
    }
}

}  // namespace

template <typename T>
cudaError_t launch_eisenstat(const PcgArgs<T>& a, LaunchShape& shape, cudaStream_t s) {
    if (shape.threads <= 0) shape.threads = kThreads;
    if (shape.lanes <= 0) shape.lanes = 1;
    const void* fn = eisenstat_fn<T>(shape.lanes);
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, shape.threads, 0)) != cudaSuccess) return e;
    const int maxb = sms * per_sm;
    if (maxb <= 0) return cudaErrorInvalidConfiguration;
    const long long want = ((long long)a.n * shape.lanes + shape.threads - 1) / shape.threads;
    int b = shape.blocks > 0 ? shape.blocks : (int)(want < maxb ? want : maxb);
    if (b > maxb) b = maxb;
    if (b < 1) b = 1;
    shape.blocks = b;
    PcgArgs<T> copy = a;
    void* args[] = {&copy};
    note_launch();
    return cudaLaunchCooperativeKernel(fn, dim3(shape.blocks), dim3(shape.threads), args, 0, s);
}

template cudaError_t launch_eisenstat<double>(const PcgArgs<double>&, LaunchShape&, cudaStream_t);
template cudaError_t launch_eisenstat<float>(const PcgArgs<float>&, LaunchShape&, cudaStream_t);

}  // namespace feec
