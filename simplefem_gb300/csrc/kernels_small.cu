// SSOR / multicolor SSOR preconditioned CG for small systems in one thread block, with
// the vectors the sweeps gather (d, m, z) held in shared memory.
//
// ConjugateGradientSolverCSR_SSOR (solver/sparsesolver.cpp:446-724) sweeps its rows in
// index order; over a dependency-level schedule that is 2 x (number of levels) dependent
// phases per iteration (129 levels on the 2D P1 operator refined 6 times). A phase then
// holds a few dozen rows, so its cost is its latency: the grid-wide or global-memory
// version pays an L2 round trip for the gathered values plus a barrier per phase. Here
// the gathered vectors live in shared memory, the barrier is the block barrier, and the
// row data of each phase (matrix entries, r, q, x, the sweep factors) is loaded several
// phases ahead: a phase costs a few shared-memory accesses and one __syncthreads. The
// arithmetic and its order per row are those of pcg_persistent (same preconditioner,
// same stopping rule, same skipped rows); only the dot products are summed by one block
// instead of a grid, and the backward sweep's z.r is summed after the sweep. When the
// phases average at most 64 rows (index-order levels), one warp walks each sweep with a
// __syncwarp between phases and the rest of the block joins in between the sweeps.
#include <cmath>
#include <cstdio>

#include "feec_device.cuh"
#include "feec_internal.h"
#include "persistent_common.cuh"

namespace feec {
namespace {

constexpr int kSmallPF = 4;   // entries of a row segment prefetched per lane
constexpr int kRing = 4;      // rows (product) or phases (sweeps) loaded ahead per group

struct SmallRow {
    int i, a, e;               // row (-1: none), segment [a, e) of the part the phase reads
    int c[kSmallPF];
    double v[kSmallPF];
    double r, q, x, w, s;      // row-local values the phase needs
};

enum { kSmFull = 0, kSmForward = 1, kSmBackward = 2 };

// Loads everything a phase needs of row slot k (k >= hi: no row) that does not depend on
// the phases before it: the matrix entries of its segment, its sweep factors and, for a
// forward row, its own r, q and x (written only by the row itself, and q by the product
// before the sweep). A backward row's r is not loaded: the backward sweep's first phase
// is loaded while the forward sweep still writes r, so z.r is summed after the sweep.
template <int KIND, int LANES>
__device__ __forceinline__ SmallRow small_row(const PcgArgs<double>& a, int k, int hi) {
    SmallRow R;
    R.i = -1; R.a = 0; R.e = 0; R.r = 0.0; R.q = 0.0; R.x = 0.0; R.w = 0.0; R.s = 0.0;
    if (k < hi) {
        if (KIND == kSmBackward) {
            R.i = __ldg(&a.brows[k]);
            R.a = __ldg(&a.usplit[R.i]);
            R.e = __ldg(&a.rp[R.i + 1]);
        } else {
            R.i = k;
            R.a = __ldg(&a.rp[k]);
            R.e = (KIND == kSmForward) ? __ldg(&a.lsplit[k]) : __ldg(&a.rp[k + 1]);
        }
        R.w = __ldg(&a.wd[R.i]);
        if (KIND == kSmForward) { R.r = a.r[R.i]; R.q = a.q[R.i]; R.x = a.x[R.i]; }
        if (KIND == kSmBackward) R.s = __ldg(&a.sd[R.i]);
    }
    const int lane = threadIdx.x & (LANES - 1);
    #pragma unroll
    for (int t = 0; t < kSmallPF; t++) {
        const int j = R.a + lane + t * LANES;
        const bool ok = j < R.e;
        R.c[t] = ok ? __ldg(&a.ci[j]) : 0;
        R.v[t] = ok ? __ldg(&a.val[j]) : 0.0;
    }
    return R;
}

// Segment dot with the gathered vector in shared memory: the same terms in the same order
// per lane as seg_dot, then the same shuffle tree.
template <int LANES>
__device__ __forceinline__ double small_dot(const SmallRow& R, const PcgArgs<double>& a, const double* sx) {
    const int lane = threadIdx.x & (LANES - 1);
    double s = 0.0;
    #pragma unroll
    for (int t = 0; t < kSmallPF; t++)
        if (R.a + lane + t * LANES < R.e) s = fma(R.v[t], sx[R.c[t]], s);
    for (int j = R.a + lane + kSmallPF * LANES; j < R.e; j += LANES) s = fma(__ldg(&a.val[j]), sx[__ldg(&a.ci[j])], s);
    #pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off, LANES);
    return s;
}

// Walks the row slots [lo, hi) of one phase (LANES lanes per row; the trip count is uniform
// across each warp for the shuffles). `cur` holds the group's first row, loaded ahead;
// each later row is loaded while the one before it is processed. A warp without a row in
// the phase branches around the body: a level holds a few dozen rows, and GB300 issues a
// warp's FP64 instruction for 16 cycles of the SM's FP64 pipe even with every lane masked
// (the idle warps' masked FP64 work was a third of the kernel's time).
template <int KIND, int LANES, int THREADS, typename F>
__device__ __forceinline__ void small_phase(const PcgArgs<double>& a, int lo, int hi, SmallRow cur, F&& body) {
    constexpr int groups = THREADS / LANES;
    const int g = threadIdx.x / LANES;
    for (int base = lo; base < hi; base += groups) {
        const SmallRow nxt = small_row<KIND, LANES>(a, base + groups + g, hi);
        if (__any_sync(0xffffffffu, cur.i >= 0)) body(cur);
        cur = nxt;
    }
}

// Rows [lo, hi) without dependences between them (the full-row product): each group keeps
// kRing of its rows in flight.
template <int KIND, int LANES, int THREADS, typename F>
__device__ __forceinline__ void small_rows_ring(const PcgArgs<double>& a, int lo, int hi, F&& body) {
    constexpr int groups = THREADS / LANES;
    const int g = threadIdx.x / LANES;
    SmallRow buf[kRing];
    #pragma unroll
    for (int k = 0; k < kRing; k++) buf[k] = small_row<KIND, LANES>(a, lo + k * groups + g, hi);
    for (int base = lo; base < hi; base += kRing * groups) {
        #pragma unroll
        for (int k = 0; k < kRing; k++) {
            if (base + k * groups < hi) {   // uniform across the warp
                body(buf[k]);
                buf[k] = small_row<KIND, LANES>(a, base + (k + kRing) * groups + g, hi);
            }
        }
    }
}

// The first row slot of the group in phase p of a sweep (forward: rows fptr[p].., backward:
// slots bptr[p]..); no row past the last phase.
template <int KIND, int LANES>
__device__ __forceinline__ SmallRow sweep_first(const PcgArgs<double>& a, int p) {
    const int g = threadIdx.x / LANES;
    if (KIND == kSmForward) {
        if (p >= a.nf) return small_row<KIND, LANES>(a, 0, 0);
        return small_row<KIND, LANES>(a, __ldg(&a.fptr[p]) + g, __ldg(&a.fptr[p + 1]));
    }
    if (p >= a.nbw) return small_row<KIND, LANES>(a, 0, 0);
    return small_row<KIND, LANES>(a, __ldg(&a.bptr[p]) + g, __ldg(&a.bptr[p + 1]));
}

// A sweep of dependent phases, one block barrier after each: the group's first row in phase
// p + kRing is loaded while phase p runs, so a phase waits for its shared-memory gathers and
// the barrier only. `ring` arrives holding the first kRing phases.
template <int KIND, int LANES, int THREADS, typename F>
__device__ __forceinline__ void small_sweep(const PcgArgs<double>& a, SmallRow (&ring)[kRing], F&& body) {
    const int nph = KIND == kSmForward ? a.nf : a.nbw;
    for (int p0 = 0; p0 < nph; p0 += kRing) {
        #pragma unroll
        for (int k = 0; k < kRing; k++) {
            const int p = p0 + k;
            if (p < nph) {   // uniform
                const int lo = KIND == kSmForward ? __ldg(&a.fptr[p]) : __ldg(&a.bptr[p]);
                const int hi = KIND == kSmForward ? __ldg(&a.fptr[p + 1]) : __ldg(&a.bptr[p + 1]);
                small_phase<KIND, LANES, THREADS>(a, lo, hi, ring[k], body);
                ring[k] = sweep_first<KIND, LANES>(a, p + kRing);
                __syncthreads();
            }
        }
    }
}

// ---- sweeps by one warp, for phases of a few dozen rows ----
// Index-order SSOR levels hold a few dozen rows (2D P1 refined 6 times: 129 levels of 33
// rows on average), so a level costs the latency of one warp's instruction path. One warp
// walks a sweep's phases with a __syncwarp between them instead of a block barrier; lane
// l takes rows l, l + 32, l + 64 of a phase and sums each row's triangular part in CSR
// order (one lane per row, the order of the reference's loop). Each row of a sweep has a
// 64-byte record in sweep order (row, first three columns and values of its triangular
// part, sweep factor), so a phase's records are one contiguous range: the warp copies the
// ranges of the next phases into a shared-memory ring with 16-byte cp.async copies, which
// the barriers do not wait for (row data loaded into registers ahead of the barriers did
// not shorten the phases: the barriers' memory ordering holds the warp until it arrives).
// The base of a row (r in
// the forward sweep, the scaled m in the backward sweep) is in shared memory: the x, r
// update writes r into z's storage, which holds nothing live until the backward sweep.
struct SweepRecord {    // 64 bytes
    int i, a, cnt;      // row, start and length of its triangular segment
    int c[3];           // first three columns (0 past cnt)
    double v[3];        // first three values (0 past cnt)
    double w;           // sweep factor
    double pad;
};
constexpr int kStageSlots = 3;                    // rows per lane per phase staged (phases of up to 96 rows)
constexpr int kStages = 4;                        // ring depth: phases in flight
constexpr int kStageRows = kStageSlots * 32;
constexpr int kRingDoubles = kStages * kStageRows * (int)sizeof(SweepRecord) / 8;

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Copies the records of phase p (at most kStageRows of them) into `st` (one commit group,
// possibly empty).
__device__ __forceinline__ void stage_phase(const SweepRecord* rec, const int* ptr, int nph, int p, SweepRecord* st,
                                            int lane) {
    if (p < nph) {
        const int lo = ptr[p];
        const int rows = min(ptr[p + 1] - lo, kStageRows);
        const char* src = reinterpret_cast<const char*>(rec + lo);
        char* dst = reinterpret_cast<char*>(st);
        for (int q = lane; q < 4 * rows; q += 32) cp_async16(dst + 16 * q, src + 16 * q);
    }
    cp_async_commit();
}

__device__ __forceinline__ void sweep_record(const SweepRecord& R, const PcgArgs<double>& a, double* x,
                                             const double* base) {
    double s = 0.0;
    #pragma unroll
    for (int u = 0; u < 3; u++)
        if (u < R.cnt) s = fma(R.v[u], x[R.c[u]], s);
    for (int j = R.a + 3; j < R.a + R.cnt; j++) s = fma(__ldg(&a.val[j]), x[__ldg(&a.ci[j])], s);
    if (R.w != 0.0) x[R.i] = (base[R.i] - s) * R.w;
}

// A whole sweep by the calling warp over the records `rec` (in sweep order, phases
// [ptr[p], ptr[p + 1])): x[i] = (base[i] - sum_j A_ij x[j]) * w.
__device__ __forceinline__ void warp_sweep(const PcgArgs<double>& a, const SweepRecord* rec, const int* ptr, int nph,
                                           double* x, const double* base, SweepRecord* ring) {
    const int lane = threadIdx.x & 31;
    #pragma unroll
    for (int q = 0; q < kStages - 1; q++) stage_phase(rec, ptr, nph, q, ring + q * kStageRows, lane);
    for (int p = 0; p < nph; p++) {
        stage_phase(rec, ptr, nph, p + kStages - 1, ring + ((p + kStages - 1) % kStages) * kStageRows, lane);
        cp_async_wait<kStages - 1>();   // this lane's copies of phase p have landed ...
        __syncwarp();                   // ... and every other lane's
        const SweepRecord* st = ring + (p % kStages) * kStageRows;
        const int lo = ptr[p], hi = ptr[p + 1];
        #pragma unroll
        for (int t = 0; t < kStageSlots; t++) {
            const int k = lane + 32 * t;
            if (lo + k < hi) sweep_record(st[k], a, x, base);
        }
        for (int k = lo + lane + kStageRows; k < hi; k += 32) sweep_record(rec[k], a, x, base);   // past the ring
        __syncwarp();   // this phase's results before the next phase gathers them
    }
    cp_async_wait<0>();
    __syncwarp();
}

// One record per row of each sweep: forward slot k is row k (the phases are row ranges),
// backward slot k is row brows[k].
__global__ void build_sweep_records(PcgArgs<double> a, SweepRecord* fwd, SweepRecord* bwd) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n) return;
    #pragma unroll
    for (int dir = 0; dir < 2; dir++) {
        const int i = dir == 0 ? k : __ldg(&a.brows[k]);
        const int lo = dir == 0 ? __ldg(&a.rp[i]) : __ldg(&a.usplit[i]);
        const int hi = dir == 0 ? __ldg(&a.lsplit[i]) : __ldg(&a.rp[i + 1]);
        SweepRecord R;
        R.i = i; R.a = lo; R.cnt = hi - lo;
        #pragma unroll
        for (int u = 0; u < 3; u++) {
            const bool ok = lo + u < hi;
            R.c[u] = ok ? __ldg(&a.ci[lo + u]) : 0;
            R.v[u] = ok ? __ldg(&a.val[lo + u]) : 0.0;
        }
        R.w = __ldg(&a.wd[i]);
        R.pad = 0.0;
        (dir == 0 ? fwd : bwd)[k] = R;
    }
}

__device__ __forceinline__ double small_block_sum(double v) {
    double vv[1] = {v};
    block_reduce<double, 1>(vv);
    __shared__ double s_sum;
    if (threadIdx.x == 0) s_sum = vv[0];
    __syncthreads();
    const double out = s_sum;
    __syncthreads();
    return out;
}

template <int LANES, int THREADS, bool WARP>
__global__ void __launch_bounds__(THREADS) pcg_smem_kernel(PcgArgs<double> a) {
    extern __shared__ __align__(16) double smem[];
    const int n = a.n;
    double* vec = WARP ? smem + kRingDoubles : smem;   // one-warp sweeps: the staging ring first
    double* sdv = vec;           // d
    double* smv = vec + n;       // m
    double* szv = vec + 2 * n;   // z
    const int lane = threadIdx.x & (LANES - 1);
    const int g = threadIdx.x / LANES;
    constexpr int groups = THREADS / LANES;
    __shared__ double s_scal[2];
    __shared__ int s_ctl;

    for (int i = threadIdx.x; i < 3 * n; i += THREADS) vec[i] = 0.0;   // work vectors start at 0
    SweepRecord* stage_ring = reinterpret_cast<SweepRecord*>(smem);
    const SweepRecord* frec = reinterpret_cast<const SweepRecord*>(a.sweep_fwd);
    const SweepRecord* brec = reinterpret_cast<const SweepRecord*>(a.sweep_bwd);
    const int* sfptr = nullptr;
    const int* sbptr = nullptr;
    if constexpr (WARP) {
        // the phase bounds of both sweeps follow the vectors
        int* sfp = reinterpret_cast<int*>(vec + 3 * n);
        int* sbp = sfp + a.nf + 1;
        for (int i = threadIdx.x; i <= a.nf; i += THREADS) sfp[i] = __ldg(&a.fptr[i]);
        for (int i = threadIdx.x; i <= a.nbw; i += THREADS) sbp[i] = __ldg(&a.bptr[i]);
        sfptr = sfp;
        sbptr = sbp;
    }
    __syncthreads();

    // ---- restart (sparsesolver.cpp:506-588): r = b - A x for rows with D != 0 ----
    double arr = 0.0;
    for (int base = 0; base < n; base += groups) {
        const int i = base + g;
        const bool act = i < n;
        const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
        double s = 0.0;
        for (int j = lo + lane; j < hi; j += LANES) s = fma(__ldg(&a.val[j]), a.x[__ldg(&a.ci[j])], s);
        #pragma unroll
        for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off, LANES);
        if (act && lane == 0 && __ldg(&a.wd[i]) != 0.0) {
            const double ri = __ldg(&a.b[i]) - s;
            a.r[i] = ri;
            if constexpr (WARP) szv[i] = ri;   // the forward sweep's base
            arr += ri * ri;
        }
    }
    __syncthreads();   // orders the r writes before the sweeps read them
    double azr = 0.0;
    if constexpr (WARP) {
        if (threadIdx.x < 32) warp_sweep(a, frec, sfptr, a.nf, smv, szv, stage_ring);
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += THREADS)
            if (__ldg(&a.wd[i]) != 0.0) smv[i] *= __ldg(&a.sd[i]);
        __syncthreads();
        if (threadIdx.x < 32) warp_sweep(a, brec, sbptr, a.nbw, szv, smv, stage_ring);
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += THREADS)
            if (__ldg(&a.wd[i]) != 0.0) {
                const double zi = szv[i];
                sdv[i] = zi;
                azr += zi * a.r[i];
            }
    } else {
        for (int p = 0; p < a.nf; p++) {                          // forward sweep
            const int lo_r = __ldg(&a.fptr[p]), hi_r = __ldg(&a.fptr[p + 1]);
            for (int base = lo_r; base < hi_r; base += groups) {
                const int i = base + g;
                const bool act = i < hi_r;
                const SmallRow R = small_row<kSmForward, LANES>(a, i, hi_r);
                const double s = small_dot<LANES>(R, a, smv);
                if (act && lane == 0) {
                    const double w = __ldg(&a.wd[i]);
                    if (w != 0.0) smv[i] = (a.r[i] - s) * w;
                }
            }
            __syncthreads();
        }
        for (int p = 0; p < a.nbw; p++) {                         // scale + backward sweep
            const int lo_r = __ldg(&a.bptr[p]), hi_r = __ldg(&a.bptr[p + 1]);
            for (int base = lo_r; base < hi_r; base += groups) {
                const int k = base + g;
                const bool act = k < hi_r;
                const SmallRow R = small_row<kSmBackward, LANES>(a, k, hi_r);
                const double s = small_dot<LANES>(R, a, szv);
                if (act && lane == 0) {
                    const double w = __ldg(&a.wd[R.i]);
                    if (w != 0.0) {
                        const double mi = smv[R.i] * __ldg(&a.sd[R.i]);
                        smv[R.i] = mi;
                        const double zi = (mi - s) * w;
                        szv[R.i] = zi;
                        sdv[R.i] = zi;
                        azr += zi * a.r[R.i];
                    }
                }
            }
            __syncthreads();
        }
    }
    double z_r = small_block_sum(azr);
    double r_r = small_block_sum(arr);

    int K = 0;
    int status = FEEC_MAXITER;
    double d_Ad = 0.0;
    SmallRow ring[kRing];
    while (K < a.max_iter) {
        if (threadIdx.x == 0) {
            if (a.print_modulo > 0 && K % a.print_modulo == 0)
                printf("(%d/%d)   INTERIM: Residual norm is %.9le < %.9le\n", K, n, sqrt(z_r), a.print_tol);
            int ctl = 0;
            if (a.use_zr_rule && fabs(z_r) < a.tol2) ctl = 1;                         // :601-604
            if (a.rr_stop > 0.0 && r_r < a.rr_stop) ctl = 1;
            s_ctl = ctl;
        }
        __syncthreads();
        if (s_ctl) { status = FEEC_OK; break; }

        double adq = 0.0;                                                            // :614-628
        small_rows_ring<kSmFull, LANES, THREADS>(a, 0, n, [&](const SmallRow& R) {
            const double s = small_dot<LANES>(R, a, sdv);
            if (R.i >= 0 && lane == 0) {
                const double qi = (R.w != 0.0) ? s : 0.0;
                a.q[R.i] = qi;
                adq += sdv[R.i] * qi;
            }
        });
        d_Ad = small_block_sum(adq);    // its barriers also order q before the forward sweep reads it
        if constexpr (!WARP) {
            #pragma unroll
            for (int k = 0; k < kRing; k++) ring[k] = sweep_first<kSmForward, LANES>(a, k);
        }
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

        const double alpha = s_scal[0];
        arr = 0.0;
        if constexpr (WARP) {
            // :640-667, the update of x and r first (rows with D != 0), then the sweep
            for (int i = threadIdx.x; i < n; i += THREADS)
                if (__ldg(&a.wd[i]) != 0.0) {
                    a.x[i] = a.x[i] + alpha * sdv[i];
                    const double ri = a.r[i] - alpha * a.q[i];
                    a.r[i] = ri;
                    szv[i] = ri;   // the forward sweep's base (z's storage is free until the backward sweep)
                    arr += ri * ri;
                }
            __syncthreads();
            if (threadIdx.x < 32) warp_sweep(a, frec, sfptr, a.nf, smv, szv, stage_ring);
            __syncthreads();
            for (int i = threadIdx.x; i < n; i += THREADS)                            // :670-699
                if (__ldg(&a.wd[i]) != 0.0) smv[i] *= __ldg(&a.sd[i]);
            __syncthreads();
            if (threadIdx.x < 32) warp_sweep(a, brec, sbptr, a.nbw, szv, smv, stage_ring);
            __syncthreads();
        } else {
            small_sweep<kSmForward, LANES, THREADS>(a, ring, [&](const SmallRow& R) {             // :640-667
                const double s = small_dot<LANES>(R, a, smv);
                if (R.i >= 0 && lane == 0 && R.w != 0.0) {
                    a.x[R.i] = R.x + alpha * sdv[R.i];
                    const double ri = R.r - alpha * R.q;
                    a.r[R.i] = ri;
                    arr += ri * ri;
                    smv[R.i] = (ri - s) * R.w;
                }
            });
            #pragma unroll
            for (int k = 0; k < kRing; k++) ring[k] = sweep_first<kSmBackward, LANES>(a, k);
            small_sweep<kSmBackward, LANES, THREADS>(a, ring, [&](const SmallRow& R) {            // :670-699
                const double s = small_dot<LANES>(R, a, szv);
                if (R.i >= 0 && lane == 0 && R.w != 0.0) {
                    const double mi = smv[R.i] * R.s;
                    smv[R.i] = mi;
                    const double zi = (mi - s) * R.w;
                    szv[R.i] = zi;
                }
            });
        }
        double azr2 = 0.0;
        for (int i = threadIdx.x; i < n; i += THREADS)                           // z.r, :690-697
            if (__ldg(&a.wd[i]) != 0.0) azr2 += szv[i] * a.r[i];
        // the block sums' barriers order x, r and z before the direction update and the next product
        const double z_r_new = small_block_sum(azr2);
        r_r = small_block_sum(arr);
        const double beta = z_r_new / z_r;                                             // :701-706
        z_r = z_r_new;
        for (int i = threadIdx.x; i < n; i += THREADS)
            if (__ldg(&a.wd[i]) != 0.0) sdv[i] = szv[i] + beta * sdv[i];
        __syncthreads();
        K++;
    }
    // the work vectors go back to global memory (callers may read d, z, m after a solve)
    for (int i = threadIdx.x; i < n; i += THREADS) { a.d[i] = sdv[i]; a.m[i] = smv[i]; a.z[i] = szv[i]; }
    finish(a.st, status, K, z_r, r_r);
}

size_t smem_bytes(int n) { return (size_t)3 * (size_t)n * sizeof(double); }

// The one-warp sweeps also hold the staging ring and the phase bounds of both sweeps.
size_t smem_bytes_warp(int n, int nf, int nbw) {
    return smem_bytes(n) + (size_t)kRingDoubles * 8 + sizeof(int) * ((size_t)nf + 1 + (size_t)nbw + 1);
}

template <int LANES, int THREADS, bool WARP>
cudaError_t launch_small(const PcgArgs<double>& a, cudaStream_t s) {
    const size_t bytes = WARP ? smem_bytes_warp(a.n, a.nf, a.nbw) : smem_bytes(a.n);
    cudaError_t e = cudaFuncSetAttribute(pcg_smem_kernel<LANES, THREADS, WARP>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    note_launch();
    pcg_smem_kernel<LANES, THREADS, WARP><<<1, THREADS, bytes, s>>>(a);
    return cudaGetLastError();
}

template <int LANES>
cudaError_t launch_small_threads(const PcgArgs<double>& a, int threads, bool warp_sweeps, cudaStream_t s) {
    if (warp_sweeps) return launch_small<LANES, 256, true>(a, s);
    if (threads <= 64) return launch_small<LANES, 64, false>(a, s);
    if (threads <= 128) return launch_small<LANES, 128, false>(a, s);
    return launch_small<LANES, 256, false>(a, s);
}

}  // namespace

int pcg_smem_max_rows() {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
    const int static_bytes = 2048;   // block reductions and scalars
    return (optin - static_bytes) / (3 * (int)sizeof(double));
}

// The block is as wide as the widest sweep phase needs (64, 128 or 256 threads): a phase's
// cost is its instruction path and barrier, which grow with the warps that take part, and
// the index-order levels hold a few dozen rows.
int pcg_smem_threads(int max_phase_rows, int lanes) {
    const long long need = (long long)max_phase_rows * lanes;
    return need <= 64 ? 64 : need <= 128 ? 128 : 256;
}

// Sweeps by one warp when the phases average at most 64 rows (index-order SSOR levels)
// and the staging ring and row bounds fit beside the vectors; by the whole block otherwise
// (multicolor phases of hundreds of rows).
bool pcg_smem_warp_sweeps(int n, int nf, int nbw) {
    if (nf <= 0 || n > 64 * nf) return false;
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
    return smem_bytes_warp(n, nf, nbw) + 2048 <= (size_t)optin;   // 2048: block reductions and scalars
}

size_t sweep_record_bytes(int n) { return (size_t)2 * (size_t)n * sizeof(SweepRecord); }

cudaError_t launch_build_sweep_records(const PcgArgs<double>& a, void* recs, cudaStream_t s) {
    SweepRecord* fwd = reinterpret_cast<SweepRecord*>(recs);
    note_launch();
    build_sweep_records<<<(a.n + 255) / 256, 256, 0, s>>>(a, fwd, fwd + a.n);
    return cudaGetLastError();
}

cudaError_t launch_pcg_smem(const PcgArgs<double>& a, int lanes, int threads, cudaStream_t s) {
    if (a.n <= 0 || a.n > pcg_smem_max_rows()) return cudaErrorInvalidValue;
    const bool warp = pcg_smem_warp_sweeps(a.n, a.nf, a.nbw) && a.sweep_fwd && a.sweep_bwd;
    switch (lanes) {
        case 1: return launch_small_threads<1>(a, threads, warp, s);
        case 2: return launch_small_threads<2>(a, threads, warp, s);
        case 4: return launch_small_threads<4>(a, threads, warp, s);
        default: return launch_small_threads<8>(a, threads, warp, s);
    }
}

}  // namespace feec
