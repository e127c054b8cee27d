// Host orchestration and the C ABI of libfeec_gpu.so (declared in include/feec_gpu.h).
//
// The drop-in entry points mirror solver/sparsesolver.hpp: they take the
// caller's host arrays, build a device-resident system, run one persistent
// cooperative solver launch and copy x and the residual back. The
// feec_system_* entry points keep everything on the device between calls.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "feec_device.cuh"
#include "feec_internal.h"
#include "feec_system.h"

namespace feec {

static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int residual_blocks(int n, int lanes);
cudaError_t launch_sum_f64(int n, const double* v, double* out, cudaStream_t s);

static const double kDesiredPrecision = 1.490116119384765625e-08;  // base/base.hpp:127-128, sqrt(2^-52)

namespace {

struct DeviceCtx {
    bool ready = false;
    cudaStream_t stream = nullptr;
    int sms = 0;
};

std::mutex g_ctx_mutex;
DeviceCtx g_ctx[64];

}  // namespace

int init_device(int& dev, cudaStream_t& stream) {
    if (cudaGetDevice(&dev) != cudaSuccess) return FEEC_NO_DEVICE;
    if (dev < 0 || dev >= 64) return FEEC_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_ctx_mutex);
    DeviceCtx& c = g_ctx[dev];
    if (!c.ready) {
        if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) return FEEC_CUDA_ERROR;
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            unsigned long long thr = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
        cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, dev);
        c.ready = true;
    }
    stream = c.stream;
    return FEEC_OK;
}

namespace {

double host_tolerance(int n, const double* b, double precision) {
    // solver/sparsesolver.cpp:45-48, the same serial loop
    double t = 0.0;
    for (int i = 0; i < n; i++) t += b[i] * b[i];
    t = precision * std::sqrt(t);
    return std::max(t, kDesiredPrecision);
}

}  // namespace
}  // namespace feec

using namespace feec;



namespace feec {
int sell_prepare(feec_system* s, int method);
SellView sell_view(const feec_system* s, int method);
}

namespace {

int ensure_work(feec_system* s) {
    if (s->work_ready) return FEEC_OK;
    HomeStreamScope home(s);
    s->work.stream = s->stream;
    const size_t n = (size_t)s->n;
    FEEC_TRY(s->work.alloc(s->x, n)); FEEC_TRY(s->work.alloc(s->r, n)); FEEC_TRY(s->work.alloc(s->d, n));
    FEEC_TRY(s->work.alloc(s->z, n)); FEEC_TRY(s->work.alloc(s->m, n)); FEEC_TRY(s->work.alloc(s->q, n));
    FEEC_TRY(s->work.alloc(s->b, n));
    FEEC_TRY(s->work.alloc(s->x32, n)); FEEC_TRY(s->work.alloc(s->r32, n)); FEEC_TRY(s->work.alloc(s->d32, n));
    FEEC_TRY(s->work.alloc(s->z32, n)); FEEC_TRY(s->work.alloc(s->m32, n)); FEEC_TRY(s->work.alloc(s->q32, n));
    FEEC_TRY(s->work.alloc(s->b32, n));
    // partial sums: up to 3 doubles per block of the largest co-resident grid, plus residual blocks
    int dev_sms = 0;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, s->dev);
    const size_t nblk = std::max<size_t>((size_t)dev_sms * 8, (size_t)residual_blocks(s->n, 32));
    FEEC_TRY(s->work.alloc(s->partials, 3 * nblk + 64));
    FEEC_TRY(s->work.alloc(s->scal, 16));
    FEEC_TRY(s->work.alloc(s->st, 1));
    if (!s->ev0) FEEC_TRY(cudaEventCreate(&s->ev0));
    if (!s->ev1) FEEC_TRY(cudaEventCreate(&s->ev1));
    s->work_ready = true;
    return FEEC_OK;
}

int read_status(feec_system* s, DeviceStatus& hs) {
    FEEC_TRY(cudaMemcpyAsync(&hs, s->st, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s->stream));
    FEEC_TRY(cudaStreamSynchronize(s->stream));
    return FEEC_OK;
}

cudaError_t reset_status(feec_system* s) {
    return cudaMemsetAsync(s->st, 0, sizeof(DeviceStatus), s->stream);
}

// ||v||^2 on the device, deterministic, read back to the host.
int device_norm2(feec_system* s, const double* v, double& out) {
    FEEC_TRY(launch_sum_sq_f64(s->n, v, s->scal, s->stream));
    FEEC_TRY(cudaMemcpyAsync(&out, s->scal, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    FEEC_TRY(cudaStreamSynchronize(s->stream));
    return FEEC_OK;
}

// r = b - A x (FP64, permuted layout if prepared else original CSR) and ||r||^2.
int true_residual(feec_system* s, const double* bb, const double* xx, double* rr, double& norm2, bool permuted) {
    const int* rp = permuted ? s->rp : s->A;
    const int* ci = permuted ? s->ci : s->C;
    const double* v = permuted ? s->val : s->V;
    const int nb = residual_blocks(s->n, s->lanes);
    FEEC_TRY(launch_residual_f64(s->n, rp, ci, v, bb, xx, rr, s->partials, s->lanes, s->stream));
    FEEC_TRY(launch_sum_f64(nb, s->partials, s->scal, s->stream));
    FEEC_TRY(cudaMemcpyAsync(&norm2, s->scal, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    FEEC_TRY(cudaStreamSynchronize(s->stream));
    return FEEC_OK;
}

template <typename T>
PcgArgs<T> make_pcg_args(feec_system* s, T* x, T* r, T* d, T* z, T* m, T* q, const T* b, const T* val, const T* wd,
                         const T* sd) {
    PcgArgs<T> a{};
    a.n = s->n; a.rp = s->rp; a.ci = s->ci; a.val = val; a.lsplit = s->lsplit; a.usplit = s->usplit;
    a.wd = wd; a.sd = sd; a.b = b; a.x = x; a.r = r; a.d = d; a.z = z; a.m = m; a.q = q;
    a.nf = s->nf; a.fptr = s->fptr; a.nbw = s->nbw; a.bptr = s->bptr; a.brows = s->brows;
    a.fsplit = s->fsplit; a.bsplit = s->bsplit;
    a.omega = s->omega; a.partials = s->partials; a.st = s->st;
    return a;
}

int timed_launch_pcg64(feec_system* s, const PcgArgs<double>& a, LaunchShape& shape, float& ms) {
    FEEC_TRY(reset_status(s));
    // Systems whose three gathered vectors fit one block's shared memory run in one block
    // (2D P1 refined 6 times: the index-order SSOR sweeps are 258 dependent level phases
    // per iteration, which one block with shared-memory vectors turns into block barriers
    // and shared-memory round trips).
    const bool small = s->user_blocks <= 0 && s->user_lanes <= 0 && a.n <= pcg_smem_max_rows();
    const bool warp = small && pcg_smem_warp_sweeps(a.n, a.nf, a.nbw);
    PcgArgs<double> ax = a;
    if (warp) {
        // per-row sweep records in sweep order, rebuilt for every solve (they hold omega / D)
        if (!s->sweep_rec) {
            HomeStreamScope home(s);
            FEEC_TRY(s->work.alloc(s->sweep_rec, sweep_record_bytes(a.n)));
        }
        FEEC_TRY(launch_build_sweep_records(a, s->sweep_rec, s->stream));
        ax.sweep_fwd = s->sweep_rec;
        ax.sweep_bwd = s->sweep_rec + sweep_record_bytes(a.n) / 2;
    }
    FEEC_TRY(cudaEventRecord(s->ev0, s->stream));
    if (small) {
        const double avg = (double)s->nnz / (double)(a.n > 0 ? a.n : 1);
        shape.lanes = avg <= 10.0 ? 1 : avg <= 20.0 ? 2 : avg <= 40.0 ? 4 : 8;
        shape.blocks = 1;
        shape.threads = warp ? 256 : pcg_smem_threads(s->max_phase_rows, shape.lanes);
        FEEC_TRY(launch_pcg_smem(ax, shape.lanes, shape.threads, s->stream));
    } else {
        FEEC_TRY(launch_pcg<double>(a, shape, s->stream));
    }
    FEEC_TRY(cudaEventRecord(s->ev1, s->stream));
    FEEC_TRY(cudaEventSynchronize(s->ev1));
    FEEC_TRY(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    return FEEC_OK;
}

void zero_info(feec_solve_info* info) {
    if (!info) return;
    std::memset(info, 0, sizeof(*info));
    info->true_relres = -1.0;
    info->outer_iterations = 1;
    info->error_estimate = -1.0;
}

const char* method_title(int method) {
    switch (method) {
        case FEEC_METHOD_SSOR: return "Conjugate Gradient CSR (SSOR)";
        case FEEC_METHOD_RAINBOW: return "Conjugate Gradient CSR (SSOR-Rainbow)";
        case FEEC_METHOD_SSOR_EISENSTAT: return "Conjugate Gradient CSR (SSOR-Eisenstat)";
        case FEEC_METHOD_RAINBOW_EISENSTAT: return "Conjugate Gradient CSR (SSOR-Rainbow-Eisenstat)";
        case FEEC_METHOD_DIAGONAL: return "Conjugate Gradient CSR (Diag)";
        default: return "Conjugate Gradient CSR";
    }
}

// Core solve on a prepared system. xx / bb / res: device arrays in the ORIGINAL numbering.
// tol_override > 0 replaces the tolerance of REFERENCE mode (the drop-in computes it on the host
// with the reference's own serial loop).
int solve_core(feec_system* s, int method, int mode, double* xx, const double* bb, double* res, double precision,
               int max_iter, double tol_override, int print_modulo, feec_solve_info* info) {
    const int n = s->n;
    const bool eisenstat = method == FEEC_METHOD_SSOR_EISENSTAT || method == FEEC_METHOD_RAINBOW_EISENSTAT;
    // the layout a method sweeps over: the Eisenstat variants use the SSOR / Rainbow ones
    const int layout = method == FEEC_METHOD_SSOR_EISENSTAT ? FEEC_METHOD_SSOR
                     : method == FEEC_METHOD_RAINBOW_EISENSTAT ? FEEC_METHOD_RAINBOW : method;
    const bool diagonal = method == FEEC_METHOD_DIAGONAL;
    // plain CG and the diagonally preconditioned CG run on the caller's CSR in its own numbering
    const bool cg_family = method == FEEC_METHOD_CG || diagonal;
    if (!cg_family && s->prepared != layout) return FEEC_BADARG;
    if (diagonal && !s->precon) return FEEC_BADARG;
    if ((eisenstat || diagonal) && mode != FEEC_MODE_REFERENCE) return FEEC_BADARG;
    int st = ensure_work(s);
    if (st != FEEC_OK) return st;
    if (max_iter <= 0) max_iter = n;
    const bool permuted = !cg_family;
    const int* perm = permuted ? s->perm : nullptr;

    // bring b, x (and the caller's residual for rows the sweeps skip) into solver order
    FEEC_TRY(launch_gather_f64(n, perm, bb, s->b, s->stream));
    FEEC_TRY(launch_gather_f64(n, perm, xx, s->x, s->stream));
    if (res) FEEC_TRY(launch_gather_f64(n, perm, res, s->r, s->stream));
    else FEEC_TRY(cudaMemsetAsync(s->r, 0, sizeof(double) * n, s->stream));

    double bnorm2 = 0.0;
    st = device_norm2(s, s->b, bnorm2);
    if (st != FEEC_OK) return st;
    const double bnorm = std::sqrt(bnorm2);
    double tolerance = tol_override > 0.0 ? tol_override : std::max(precision * bnorm, kDesiredPrecision);
    if (mode != FEEC_MODE_REFERENCE) tolerance = precision * bnorm;

    // MIXED on the whole GPU: a system measures its first solve with FP32 inner iterations
    // and its second with FP64 ones (device time per decade of residual fall) and keeps the
    // faster for later solves of the same method. The phases of a single solve are latency-
    // bound, so FP32 storage may not pay for its extra iterations (3D P1 refined 7 times:
    // 223 ms against 168 in FP64); the result reports the choice in inner_fp64.
    const int pick_slot = method == FEEC_METHOD_CG ? 0 : 1;
    bool inner64 = false;
    if (mode == FEEC_MODE_MIXED) {
        const int pick = s->mixed_pick[pick_slot];
        inner64 = pick == 2 || (pick == 0 && s->mixed_rate[pick_slot][0] > 0.0);
    }
    const int shape_mode = inner64 ? FEEC_MODE_FP64 : mode;

    LaunchShape shape;
    shape.lanes = s->lanes;
    // Measured on GB300 (3D P2 operator, 28 entries per row, two 512-thread blocks per
    // SM): the FP64 persistent solvers issue FP64 at 2 lanes/clk/SM, so wide per-row
    // reductions and per-group epilogues cost more than they save; 2 lanes per row are
    // fastest for plain FP64 CG (42.7 ms against 50.4 with 1, and 47.3 with 1 lane on one
    // block per SM) and 4 for the sweeps of the preconditioned solvers (50.2 ms against
    // 56.3 with 8 and 76.0 with 16; 8 for their FP32 inner solves).
    if (cg_family && shape_mode != FEEC_MODE_MIXED) shape.lanes = 2;
    else {
        const int cap = (shape_mode == FEEC_MODE_MIXED && method != FEEC_METHOD_CG) ? 8 : 4;
        if (shape.lanes > cap) shape.lanes = cap;
    }
    if (shape.lanes == 1 || shape.lanes == 4 || shape.lanes == 8) {
        // two co-resident blocks per SM were fastest in the same measurements
        int dev_sms = 0;
        cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, s->dev);
        shape.blocks = 2 * dev_sms;
    }
    if (permuted && s->max_phase_rows > 0) {
        // one pass over the largest sweep phase: enough row groups in the co-resident grid
        const int maxb = max_coresident_blocks(1, 0, shape.lanes, 512);
        while (shape.lanes > 1 && (long long)maxb * 512 / shape.lanes < s->max_phase_rows) shape.lanes >>= 1;
    }
    // Small systems (measured on GB300, 4,225-16,641 unknowns): the index-order SSOR sweeps
    // are hundreds of dependent level phases per iteration, and a one-block grid turns each
    // grid barrier into a block barrier (2D P1 L6: 103 -> 61 ms; 2D P1 L7: 412 -> 273 ms)
    // while one SM's FP64 rate still covers the products; the other methods gain ~15 % from
    // a 16-block grid on the smallest systems.
    if (layout == FEEC_METHOD_SSOR && s->nnz <= 200000) shape.blocks = 1;
    else if (s->nnz < 60000) shape.blocks = 16;
    if (s->user_lanes > 0) shape.lanes = s->user_lanes;
    if (s->user_blocks > 0) shape.blocks = s->user_blocks;
    float ms_total = 0.0f;
    int K_total = 0, outer = 0, status = FEEC_OK;
    double final_norm = 0.0;
    int fell_back = 0;
    double err_estimate = -1.0;      // MIXED: estimated relative error of x (-1: not estimated)
    DeviceStatus hs{};

    // FP64 solve from the current iterate s->x: run with the recursive-residual rule, then
    // confirm on the true residual and restart from the current iterate if the recursion
    // drifted (at most a few times). REFERENCE mode runs once with the reference's rule.
    auto run_fp64 = [&](int run_mode) -> int {
        const int max_restarts = (run_mode == FEEC_MODE_FP64) ? 4 : 1;
        const int k0 = K_total;   // iterations before this FP64 run do not count against its budget
        for (int attempt = 0; attempt < max_restarts; attempt++) {
            FEEC_TRY(cudaMemsetAsync(s->d, 0, sizeof(double) * n, s->stream));
            FEEC_TRY(cudaMemsetAsync(s->z, 0, sizeof(double) * n, s->stream));
            FEEC_TRY(cudaMemsetAsync(s->m, 0, sizeof(double) * n, s->stream));
            FEEC_TRY(cudaMemsetAsync(s->q, 0, sizeof(double) * n, s->stream));
            float ms = 0.0f;
            if (cg_family) {
                CgArgs<double> a{};
                a.n = n; a.rp = s->A; a.ci = s->C; a.val = s->V; a.b = s->b; a.x = s->x; a.r = s->r; a.d = s->d; a.q = s->q;
                if (diagonal) {
                    a.precon = s->precon; a.z = s->z;
                    // the reference starts its work vectors as NaN (sparsesolver.cpp:259-264);
                    // rows it skips (precon == 0) keep that value
                    for (double* v : {s->d, s->z, s->q})
                        FEEC_TRY(cudaMemsetAsync(v, 0xFF, sizeof(double) * n, s->stream));
                }
                a.tol2 = tolerance * tolerance;
                a.max_iter = max_iter - (K_total - k0);
                a.print_modulo = print_modulo; a.print_tol = tolerance;
                a.partials = s->partials; a.st = s->st;
                FEEC_TRY(reset_status(s));
                FEEC_TRY(cudaEventRecord(s->ev0, s->stream));
                FEEC_TRY(launch_cg<double>(a, shape, s->stream));
                FEEC_TRY(cudaEventRecord(s->ev1, s->stream));
                FEEC_TRY(cudaEventSynchronize(s->ev1));
                FEEC_TRY(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
            } else if (eisenstat) {
                if (!s->w) {
                    HomeStreamScope home(s);
                    FEEC_TRY(s->work.alloc(s->w, (size_t)n));
                }
                // the reference starts its work vectors as NaN (sparsesolver.cpp:766-773,
                // 1383-1394); rows the sweeps skip (D == 0) keep that value
                for (double* v : {s->d, s->z, s->m, s->q, s->w})
                    FEEC_TRY(cudaMemsetAsync(v, 0xFF, sizeof(double) * n, s->stream));
                PcgArgs<double> a = make_pcg_args<double>(s, s->x, s->r, s->d, s->z, s->m, s->q, s->b, s->val, s->wd, s->sd);
                a.dg = s->diag; a.w = s->w;
                a.guard_restart = s->zero_diag_rows > 0;
                a.guard_iter = method == FEEC_METHOD_SSOR_EISENSTAT && s->zero_diag_rows > 0;
                a.tol2 = tolerance * tolerance;
                a.use_zr_rule = 1;
                a.max_iter = max_iter - (K_total - k0);
                a.print_modulo = print_modulo; a.print_tol = tolerance;
                FEEC_TRY(reset_status(s));
                FEEC_TRY(cudaEventRecord(s->ev0, s->stream));
                FEEC_TRY(launch_eisenstat<double>(a, shape, s->stream));
                FEEC_TRY(cudaEventRecord(s->ev1, s->stream));
                FEEC_TRY(cudaEventSynchronize(s->ev1));
                FEEC_TRY(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
            } else if (run_mode == FEEC_MODE_FP64) {
                // FP64 product mode of the preconditioned solvers: Eisenstat's formulation (the
                // same preconditioned iterates, no SpMV over full rows per iteration). It stops
                // when z.r has fallen by (tolerance / ||b - A x||)^2; the check below confirms
                // on the true residual and restarts from the current iterate if needed.
                double rn2 = 0.0;
                st = true_residual(s, s->b, s->x, s->q, rn2, permuted);
                if (st != FEEC_OK) return st;
                if (std::sqrt(rn2) <= tolerance) { status = FEEC_OK; final_norm = std::sqrt(rn2); break; }
                if (!s->w) {
                    HomeStreamScope home(s);
                    FEEC_TRY(s->work.alloc(s->w, (size_t)n));
                }
                PcgArgs<double> a = make_pcg_args<double>(s, s->x, s->r, s->d, s->z, s->m, s->q, s->b, s->val, s->wd, s->sd);
                a.dg = s->diag; a.w = s->w;
                a.guard_restart = a.guard_iter = s->zero_diag_rows > 0;
                a.use_zr_rule = 0;
                a.rr_stop = tolerance * tolerance / rn2;
                a.max_iter = max_iter - (K_total - k0);
                FEEC_TRY(reset_status(s));
                FEEC_TRY(cudaEventRecord(s->ev0, s->stream));
                FEEC_TRY(launch_eisenstat<double>(a, shape, s->stream));
                FEEC_TRY(cudaEventRecord(s->ev1, s->stream));
                FEEC_TRY(cudaEventSynchronize(s->ev1));
                FEEC_TRY(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
            } else {
                PcgArgs<double> a = make_pcg_args<double>(s, s->x, s->r, s->d, s->z, s->m, s->q, s->b, s->val, s->wd, s->sd);
                a.tol2 = tolerance * tolerance;
                a.use_zr_rule = (run_mode == FEEC_MODE_REFERENCE) ? 1 : 0;
                a.rr_stop = (run_mode == FEEC_MODE_FP64) ? tolerance * tolerance : 0.0;
                a.max_iter = max_iter - (K_total - k0);
                a.print_modulo = print_modulo; a.print_tol = tolerance;
                st = timed_launch_pcg64(s, a, shape, ms);
                if (st != FEEC_OK) return st;
            }
            ms_total += ms;
            st = read_status(s, hs);
            if (st != FEEC_OK) return st;
            K_total += hs.iterations;
            status = hs.status;
            final_norm = std::sqrt(std::fabs(hs.final_value));
            outer++;
            if (run_mode == FEEC_MODE_REFERENCE || status != FEEC_OK) break;
            double rn2 = 0.0;
            st = true_residual(s, s->b, s->x, s->d, rn2, permuted);
            if (st != FEEC_OK) return st;
            final_norm = std::sqrt(rn2);
            if (final_norm <= tolerance) break;
            if (K_total - k0 >= max_iter) { status = FEEC_MAXITER; break; }
        }
        return FEEC_OK;
    };

    if (mode == FEEC_MODE_REFERENCE || mode == FEEC_MODE_FP64) {
        st = run_fp64(mode);
        if (st != FEEC_OK) return st;
    } else if (inner64) {
        // MIXED with FP64 inner iterations: the residual bar tightened so that the error bar
        // holds for amplifications up to kAmpFloor (kAmpFloor x relative residual <=
        // kErrorPerResidual x precision), the bound reported as the estimate
        tolerance = precision * bnorm * kErrorPerResidual / kAmpFloor;
        st = run_fp64(FEEC_MODE_FP64);
        if (st != FEEC_OK) return st;
        if (bnorm > 0.0) err_estimate = kAmpFloor * final_norm / bnorm;
        tolerance = precision * bnorm;
    } else {
        // MIXED: FP32 inner iterations (compensated FP32 dots) in segments: the FP64 solution
        // and true residual are kept beside the FP32 recursion, and a segment ends when z.r
        // (r.r for CG) has fallen by the square of kReliableDelta (kRestartEta for CG) or far
        // enough for the target; the correction then goes into x in FP64 and the FP64 true
        // residual replaces the recursive one (scaled to unit norm). The multicolor SSOR-PCG
        // keeps its search direction across the replacement (rescaled, beta against the
        // previous rho: reliable updates) instead of restarting the Krylov recurrence; plain
        // CG restarts (plain defect correction), see kRestartEta.
        if (method == FEEC_METHOD_CG && !s->V32) return FEEC_BADARG;
        if (method != FEEC_METHOD_CG && !s->val32) return FEEC_BADARG;
        const int max_outer = kMaxReplacements;
        const bool keep_dirs = method != FEEC_METHOD_CG;   // plain CG restarts each segment
        const double seg = keep_dirs ? kReliableDelta : kRestartEta;
        const double delta2 = seg * seg;
        const double first2 = kRestartEta * kRestartEta;   // see kReliableDelta
        double rn2 = 0.0;
        double stall_limit = 0.0;        // residual norm above which the last segment stagnated
        bool stagnated = false;
        // Error control. A small residual does not make a small error: what the FP32 inner
        // iterations leave behind is mostly smooth, low-eigenvalue error, which A shrinks the
        // most. Each segment measures how large its correction was against the residual it
        // corrected (the correction approximates the error of the iterate it corrected),
        // which gives the error-to-residual amplification of this operator; the solve then
        // also asks max(amplification, kAmpFloor) x relative residual <= err_target before
        // it stops, and sizes each segment's target for both bars.
        const double err_target = kErrorPerResidual * precision;
        double amp = 0.0;                // largest measured amplification (segments after the first)
        bool err_step = false;           // the residual bar is met, the error bar not yet
        bool have_dir = false;           // a search direction to keep from the last segment
        bool keep_live = keep_dirs;      // cleared once a kept direction stops paying
        // Iterations per decade of z.r fall of the restarted segments (the largest seen). A
        // kept direction stays consistent with the replaced residual only while the FP32
        // recursion's drift within a segment is small against that residual; on operators
        // whose condition number times the FP32 unit roundoff nears 1e-2 it is not, and the
        // kept segments slow down without bound (2D P1 refined 10 times: 0.7 k, 1.1 k, 14 k,
        // 60 k, 258 k iterations for the same 0.01 fall). A kept segment is therefore given
        // at most kKeptSegmentSlack times the restarted rate for its fall; one that runs out
        // ends there, and every later segment restarts.
        double restart_rate = 0.0;
        double zr_prev = 0.0, rn_prev = 0.0;
        for (outer = 0; outer < max_outer; outer++) {
            st = true_residual(s, s->b, s->x, s->r, rn2, permuted);
            if (st != FEEC_OK) return st;
            const double rn = std::sqrt(rn2);
            final_norm = rn;
            if (!(rn == rn)) { status = FEEC_BREAKDOWN; break; }
            const double relres = bnorm > 0.0 ? rn / bnorm : 0.0;
            if (rn <= tolerance) {
                // stop at the error bar, or when the residual no longer falls (the FP64
                // residual's own rounding floor) after the bar was first missed
                const bool floor = err_step && rn > 0.3 * rn_prev;
                if (std::max(amp, kAmpFloor) * relres <= err_target || floor || K_total >= max_iter) {
                    status = FEEC_OK;
                    break;
                }
                err_step = true;
            }
            // A segment whose true residual gained less than half the digits its recursion
            // promised means the operator is too ill-conditioned for FP32 arithmetic
            // (condition number times the FP32 unit roundoff near 1e-2 or above): finish in
            // FP64 from the current iterate, with a fresh budget of max_iter iterations.
            if (outer > 0 && rn > stall_limit && rn > tolerance) { stagnated = true; break; }
            if (K_total >= max_iter) { status = FEEC_MAXITER; break; }
            const double scale = (have_dir && rn > 0.0) ? rn_prev / rn : 1.0;
            const double inv = 1.0 / rn;
            const double scal_h[2] = {inv, rn};
            FEEC_TRY(cudaMemcpyAsync(s->scal + 2, scal_h, sizeof(scal_h), cudaMemcpyHostToDevice, s->stream));
            FEEC_TRY(launch_scaled_cast(n, s->r, s->scal + 2, s->b32, s->stream));
            FEEC_TRY(cudaMemsetAsync(s->x32, 0, sizeof(float) * n, s->stream));
            if (!have_dir) {
                FEEC_TRY(cudaMemsetAsync(s->d32, 0, sizeof(float) * n, s->stream));
                FEEC_TRY(cudaMemsetAsync(s->z32, 0, sizeof(float) * n, s->stream));
                FEEC_TRY(cudaMemsetAsync(s->m32, 0, sizeof(float) * n, s->stream));
                FEEC_TRY(cudaMemsetAsync(s->q32, 0, sizeof(float) * n, s->stream));
                FEEC_TRY(cudaMemsetAsync(s->r32, 0, sizeof(float) * n, s->stream));
            }
            // the segment's target: the residual bar and, once an amplification is known, the
            // error bar (with margin), or a fall of kReliableDelta, whichever comes first
            // (the larger of the two factors)
            const double target = std::min(tolerance, err_target * bnorm / std::max(amp, kAmpFloor));
            const double need = 0.3 * target / rn;
            const double f = std::max(outer == 0 ? first2 : delta2, need * need);
            stall_limit = rn * std::sqrt(std::sqrt(f));
            const double decades = std::max(1.0, -std::log10(f));
            int seg_budget = max_iter - K_total;
            if (have_dir && restart_rate > 0.0) {
                const double cap = kKeptSegmentSlack * restart_rate * decades + 32.0;
                if (cap < (double)seg_budget) seg_budget = (int)cap;
            }
            float ms = 0.0f;
            FEEC_TRY(reset_status(s));
            FEEC_TRY(cudaEventRecord(s->ev0, s->stream));
            if (method == FEEC_METHOD_CG) {
                CgArgs<float> a{};
                a.n = n; a.rp = s->A; a.ci = s->C; a.val = s->V32; a.b = s->b32; a.x = s->x32; a.r = s->r32;
                a.d = s->d32; a.q = s->q32;
                a.tol2 = f;                       // r starts at unit norm: a relative fall of f in r.r
                a.max_iter = seg_budget;
                a.partials = s->partials; a.st = s->st;
                a.keep_dir = have_dir ? 1 : 0; a.zr_prev = zr_prev; a.scale = scale;
                FEEC_TRY(launch_cg<float>(a, shape, s->stream));
            } else {
                // The inner multicolor / index-order SSOR-PCG runs in Eisenstat's formulation:
                // the same preconditioned iterates, but an iteration is one backward and one
                // forward sweep over the strict parts, with no SpMV over full rows.
                if (!s->w32) {
                    HomeStreamScope home(s);
                    FEEC_TRY(s->work.alloc(s->w32, (size_t)n));
                }
                PcgArgs<float> a = make_pcg_args<float>(s, s->x32, s->r32, s->d32, s->z32, s->m32, s->q32, s->b32,
                                                        s->val32, s->wd32, s->sd32);
                a.dg = s->diag32; a.w = s->w32;
                a.guard_restart = a.guard_iter = s->zero_diag_rows > 0;
                a.use_zr_rule = 0;
                a.rr_stop = f;
                a.max_iter = seg_budget;
                a.keep_dir = have_dir ? 1 : 0; a.zr_prev = zr_prev; a.scale = scale;
                FEEC_TRY(launch_eisenstat<float>(a, shape, s->stream));
            }
            FEEC_TRY(cudaEventRecord(s->ev1, s->stream));
            FEEC_TRY(launch_update_x_norms(n, s->x32, s->scal + 3, s->x, s->partials, s->scal + 4, s->stream));
            double norms2[2] = {0.0, 0.0};   // ||correction||^2, ||x||^2
            FEEC_TRY(cudaMemcpyAsync(norms2, s->scal + 4, sizeof(norms2), cudaMemcpyDeviceToHost, s->stream));
            FEEC_TRY(cudaEventSynchronize(s->ev1));
            FEEC_TRY(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
            FEEC_TRY(cudaStreamSynchronize(s->stream));
            ms_total += ms;
            st = read_status(s, hs);
            if (st != FEEC_OK) return st;
            K_total += hs.iterations;
            // the first segment starts from the initial guess (its correction is the
            // solution); a later one measures the error of the iterate it corrected
            if (outer > 0 && norms2[1] > 0.0 && relres > 0.0)
                amp = std::max(amp, std::sqrt(norms2[0] / norms2[1]) / relres);
            if (hs.status == FEEC_TIMEOUT) { status = FEEC_TIMEOUT; break; }
            if (hs.status == FEEC_BREAKDOWN && hs.iterations == 0) { status = FEEC_BREAKDOWN; break; }
            if (!have_dir && hs.status == FEEC_OK && hs.iterations > 0)
                restart_rate = std::max(restart_rate, hs.iterations / decades);
            if (have_dir && hs.status == FEEC_MAXITER && hs.iterations >= seg_budget &&
                seg_budget < max_iter - (K_total - hs.iterations)) {
                // a kept segment that ran out of its share: restart from here on; its true
                // residual only has to fall (it did not reach the fall it was asked for)
                keep_live = false;
                stall_limit = rn;
            }
            // a breakdown or an empty segment restarts the direction next time
            // (and the long first segment's direction, whose recursion drifted too far from the
            // true residual to fit the replaced one)
            have_dir = keep_live && outer > 0 && hs.status == FEEC_OK && hs.iterations > 0;
            zr_prev = hs.extra[0];
            rn_prev = rn;
        }
        if (outer == max_outer) status = FEEC_MAXITER;
        if (stagnated) {
            st = run_fp64(FEEC_MODE_FP64);
            if (st != FEEC_OK) return st;
            fell_back = 1;
        }
        // leave the FP64 recursive residual array holding the true residual
        double rn2b = 0.0;
        st = true_residual(s, s->b, s->x, s->r, rn2b, permuted);
        if (st != FEEC_OK) return st;
        final_norm = std::sqrt(rn2b);
        if (status == FEEC_OK && final_norm > tolerance) status = FEEC_MAXITER;
        // the bound the stop rule enforced: max(amplification, kAmpFloor) x relative residual
        if (!fell_back && bnorm > 0.0) err_estimate = std::max(amp, kAmpFloor) * final_norm / bnorm;
    }

    if (mode == FEEC_MODE_MIXED && s->mixed_pick[pick_slot] == 0 && status == FEEC_OK && final_norm > 0.0 &&
        bnorm > 0.0) {
        const double decades = std::max(1.0, std::log10(bnorm / final_norm));
        s->mixed_rate[pick_slot][inner64 ? 1 : 0] = ms_total / decades;
        if (inner64) s->mixed_pick[pick_slot] = s->mixed_rate[pick_slot][1] < s->mixed_rate[pick_slot][0] ? 2 : 1;
    }

    // results back to the caller's numbering
    FEEC_TRY(launch_scatter_f64(n, perm, s->x, xx, s->stream));
    if (res) FEEC_TRY(launch_scatter_f64(n, perm, s->r, res, s->stream));

    if (info) {
        info->status = status;
        info->iterations = K_total;
        info->outer_iterations = outer;
        info->num_colors = cg_family ? 0 : s->num_levels;
        info->fp64_fallback = fell_back;
        info->inner_fp64 = inner64 ? 1 : 0;
        info->error_estimate = err_estimate;
        info->tolerance = (mode == FEEC_MODE_REFERENCE) ? tolerance : precision;
        info->final_norm = final_norm;
        info->device_ms = ms_total;
        info->grid_blocks = shape.blocks;
        info->lanes_per_row = shape.lanes;
        if (mode != FEEC_MODE_REFERENCE) {
            double rn2 = 0.0;
            st = true_residual(s, s->b, s->x, s->d, rn2, permuted);
            if (st != FEEC_OK) return st;
            info->true_relres = bnorm > 0 ? std::sqrt(rn2) / bnorm : 0.0;
        }
    }
    FEEC_TRY(cudaStreamSynchronize(s->stream));
    return status;
}

int build_layout(feec_system* s, int method, const double* diag_dev, double omega, const int* perm_host,
                 const int* key_dev, const std::vector<int>& fptr, const std::vector<int>& bptr,
                 const std::vector<int>& brows, int num_levels) {
    const int n = s->n;
    cudaStream_t st = s->stream;
    DevArena& M = s->mem;
    if (!s->perm) {
        FEEC_TRY(M.alloc(s->perm, n)); FEEC_TRY(M.alloc(s->iperm, n));
        FEEC_TRY(M.alloc(s->rp, (size_t)n + 1)); FEEC_TRY(M.alloc(s->ci, (size_t)s->nnz));
        FEEC_TRY(M.alloc(s->val, (size_t)s->nnz)); FEEC_TRY(M.alloc(s->val32, (size_t)s->nnz));
        FEEC_TRY(M.alloc(s->lsplit, n)); FEEC_TRY(M.alloc(s->usplit, n));
        FEEC_TRY(M.alloc(s->diag, n)); FEEC_TRY(M.alloc(s->diag32, n));
        FEEC_TRY(M.alloc(s->wd, n)); FEEC_TRY(M.alloc(s->sd, n)); FEEC_TRY(M.alloc(s->wd32, n)); FEEC_TRY(M.alloc(s->sd32, n));
    }
    // schedules (small, reallocated per preparation)
    s->fsplit = nullptr; s->bsplit = nullptr;
    FEEC_TRY(M.alloc(s->fptr, fptr.size())); FEEC_TRY(M.alloc(s->bptr, bptr.size())); FEEC_TRY(M.alloc(s->brows, brows.size()));
    FEEC_TRY(cudaMemcpyAsync(s->perm, perm_host, sizeof(int) * n, cudaMemcpyHostToDevice, st));
    FEEC_TRY(cudaMemcpyAsync(s->fptr, fptr.data(), sizeof(int) * fptr.size(), cudaMemcpyHostToDevice, st));
    FEEC_TRY(cudaMemcpyAsync(s->bptr, bptr.data(), sizeof(int) * bptr.size(), cudaMemcpyHostToDevice, st));
    FEEC_TRY(cudaMemcpyAsync(s->brows, brows.data(), sizeof(int) * brows.size(), cudaMemcpyHostToDevice, st));
    FEEC_TRY(launch_inverse_perm(n, s->perm, s->iperm, st));
    int *len = nullptr, *scratch = nullptr;
    DevArena tmp; tmp.stream = st;
    FEEC_TRY(tmp.alloc(len, (size_t)n + 1));
    FEEC_TRY(tmp.alloc(scratch, scan_scratch_ints(n + 1)));
    FEEC_TRY(cudaMemsetAsync(len + n, 0, sizeof(int), st));
    FEEC_TRY(launch_row_lengths(n, s->A, s->perm, len, st));
    FEEC_TRY(launch_exclusive_scan(n + 1, len, s->rp, scratch, st));
    FEEC_TRY(launch_permute_split(n, s->A, s->C, s->V, s->perm, s->iperm, key_dev, s->rp, s->ci, s->val, s->val32,
                                  s->lsplit, s->usplit, st));
    FEEC_TRY(launch_gather_f64(n, s->perm, diag_dev, s->diag, st));
    FEEC_TRY(launch_cast_f64_f32((size_t)n, s->diag, s->diag32, st));
    FEEC_TRY(launch_sweep_factors(n, s->diag, omega, s->wd, s->sd, s->wd32, s->sd32, st));
    tmp.release();
    {
        std::vector<double> dh((size_t)n);
        FEEC_TRY(cudaMemcpyAsync(dh.data(), s->diag, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        FEEC_TRY(cudaStreamSynchronize(st));
        s->zero_diag_rows = (int)std::count(dh.begin(), dh.end(), 0.0);
    }
    FEEC_TRY(cudaStreamSynchronize(st));
    s->nf = (int)fptr.size() - 1;
    s->nbw = (int)bptr.size() - 1;
    s->max_phase_rows = 0;
    for (size_t p = 0; p + 1 < fptr.size(); p++) s->max_phase_rows = std::max(s->max_phase_rows, fptr[p + 1] - fptr[p]);
    for (size_t p = 0; p + 1 < bptr.size(); p++) s->max_phase_rows = std::max(s->max_phase_rows, bptr[p + 1] - bptr[p]);
    s->omega = omega;
    s->num_levels = num_levels;
    s->prepared = method;
    s->mixed_pick[1] = 0;   // a new layout measures its inner precision again
    s->mixed_rate[1][0] = s->mixed_rate[1][1] = 0.0;
    s->sell[1].ready = false;   // the Rainbow-order SELL copy follows the new ordering
    return FEEC_OK;
}

int copy_in_ints(feec_system* s, const int* src, int count, int host_ptrs, std::vector<int>& out) {
    out.resize((size_t)count);
    if (count == 0) return FEEC_OK;
    FEEC_TRY(cudaMemcpyAsync(out.data(), src, sizeof(int) * count, host_ptrs ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost, s->stream));
    FEEC_TRY(cudaStreamSynchronize(s->stream));
    return FEEC_OK;
}

}  // namespace

extern "C" {

const char* feec_status_string(int status) {
    switch (status) {
        case FEEC_OK: return "ok";
        case FEEC_BREAKDOWN: return "breakdown";
        case FEEC_SMALL_ENERGY: return "small gradient energy";
        case FEEC_MAXITER: return "iteration limit";
        case FEEC_TIMEOUT: return "device wait timed out";
        case FEEC_OOM: return "out of device memory";
        case FEEC_BADARG: return "bad argument";
        case FEEC_CUDA_ERROR: return "CUDA error";
        case FEEC_NO_DEVICE: return "no device";
        default: return "unknown";
    }
}

unsigned long long feec_kernel_launches(void) { return g_launches.load(); }

int feec_system_create(feec_system** out, int N, const int* A, const int* C, const double* V, int host_ptrs, void* stream) {
    if (!out || N <= 0 || !A || !C || !V) return FEEC_BADARG;
    *out = nullptr;
    int dev = 0;
    cudaStream_t lib_stream = nullptr;
    int st = init_device(dev, lib_stream);
    if (st != FEEC_OK) return st;
    feec_system* s = new (std::nothrow) feec_system();
    if (!s) return FEEC_OOM;
    s->dev = dev;
    s->n = N;
    // NULL means CUDA's default stream (stream 0), so the system is ordered with other
    // work the caller issues there (e.g. a framework's default stream)
    (void)lib_stream;
    s->stream = (cudaStream_t)stream;
    s->home_stream = s->stream;
    s->mem.stream = s->stream;
    s->work.stream = s->stream;
    int nnz = 0;
    cudaError_t e = cudaMemcpyAsync(&nnz, A + N, sizeof(int), host_ptrs ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess || nnz < 0) { delete s; return e != cudaSuccess ? cuda_status(e) : FEEC_BADARG; }
    s->nnz = nnz;
    const cudaMemcpyKind kind = host_ptrs ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if ((e = s->mem.alloc(s->A, (size_t)N + 1)) != cudaSuccess ||
        (e = s->mem.alloc(s->C, (size_t)nnz)) != cudaSuccess ||
        (e = s->mem.alloc(s->V, (size_t)nnz)) != cudaSuccess ||
        (e = s->mem.alloc(s->V32, (size_t)nnz)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s->A, A, sizeof(int) * ((size_t)N + 1), kind, s->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s->C, C, sizeof(int) * (size_t)nnz, kind, s->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s->V, V, sizeof(double) * (size_t)nnz, kind, s->stream)) != cudaSuccess ||
        (e = launch_cast_f64_f32((size_t)nnz, s->V, s->V32, s->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s->stream)) != cudaSuccess) {
        s->mem.release();
        cudaStreamSynchronize(s->stream);
        delete s;
        return cuda_status(e);
    }
    // every column index and row pointer is checked before any kernel indexes through them
    int* bad_d = nullptr;
    int bad = 0;
    if ((e = s->mem.alloc(bad_d, 1)) != cudaSuccess || (e = cudaMemsetAsync(bad_d, 0, sizeof(int), s->stream)) != cudaSuccess ||
        (e = launch_validate_csr(N, nnz, s->A, s->C, bad_d, s->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&bad, bad_d, sizeof(int), cudaMemcpyDeviceToHost, s->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s->stream)) != cudaSuccess || bad) {
        s->mem.release();
        cudaStreamSynchronize(s->stream);
        delete s;
        return e != cudaSuccess ? cuda_status(e) : FEEC_BADARG;
    }
    s->lanes = pick_lanes((double)nnz / (double)N);
    *out = s;
    return FEEC_OK;
}

int feec_system_destroy(feec_system* s) {
    if (!s) return FEEC_OK;
    s->work.release();
    s->sell[0].mem.release();
    s->sell[1].mem.release();
    s->mem.release();
    cudaStreamSynchronize(s->stream);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    delete s;
    return FEEC_OK;
}

int feec_system_set_launch(feec_system* s, int blocks, int lanes) {
    if (!s || blocks < 0 || lanes < 0 || lanes > 32 || (lanes & (lanes - 1)) != 0) return FEEC_BADARG;
    s->user_blocks = blocks;
    s->user_lanes = lanes;
    return FEEC_OK;
}

int feec_system_memory(const feec_system* s, size_t* bytes) {
    if (!s || !bytes) return FEEC_BADARG;
    *bytes = s->mem.bytes + s->work.bytes;
    return FEEC_OK;
}

int feec_system_set_rainbow(feec_system* s, const double* diagonal, double omega, int num_colors, const int* F,
                            const int* B, const int* R, int host_ptrs) {
    if (!s || !diagonal || !F || !B || !R || num_colors < 0 || !(omega > 0.0) || !(omega < 2.0)) return FEEC_BADARG;
    const int n = s->n;
    std::vector<int> hB, hR;
    int st = copy_in_ints(s, B, num_colors + 1, host_ptrs, hB);
    if (st != FEEC_OK) return st;
    st = copy_in_ints(s, R, n, host_ptrs, hR);
    if (st != FEEC_OK) return st;
    if (hB[0] != 0 || hB[num_colors] != n) return FEEC_BADARG;
    for (int c = 0; c < num_colors; c++) if (hB[c + 1] < hB[c]) return FEEC_BADARG;
    std::vector<char> seen((size_t)n, 0);
    for (int i = 0; i < n; i++) {
        if (hR[i] < 0 || hR[i] >= n || seen[hR[i]]) return FEEC_BADARG;
        seen[hR[i]] = 1;
    }
    // Inside a color the rows are independent, so their order is free: sort them by row
    // length (stable, longest first) so that 32-row slices hold rows of equal length.
    std::vector<int> hA((size_t)n + 1);
    FEEC_TRY(cudaMemcpyAsync(hA.data(), s->A, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s->stream));
    FEEC_TRY(cudaStreamSynchronize(s->stream));
    for (int c = 0; c < num_colors; c++)
        std::stable_sort(hR.begin() + hB[c], hR.begin() + hB[c + 1],
                         [&](int a, int b) { return hA[a + 1] - hA[a] > hA[b + 1] - hA[b]; });
    // forward phases: colors ascending (rows are renumbered color by color, so ranges are contiguous);
    // backward phases: colors descending
    std::vector<int> fptr(hB.begin(), hB.end());
    std::vector<int> bptr(1, 0), brows;
    brows.reserve(n);
    for (int c = num_colors - 1; c >= 0; c--) {
        for (int i = hB[c]; i < hB[c + 1]; i++) brows.push_back(i);
        bptr.push_back((int)brows.size());
    }
    DevArena tmp; tmp.stream = s->stream;
    int* Fd = nullptr; double* Dd = nullptr;
    FEEC_TRY(tmp.alloc(Fd, n)); FEEC_TRY(tmp.alloc(Dd, n));
    const cudaMemcpyKind kind = host_ptrs ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    FEEC_TRY(cudaMemcpyAsync(Fd, F, sizeof(int) * n, kind, s->stream));
    FEEC_TRY(cudaMemcpyAsync(Dd, diagonal, sizeof(double) * n, kind, s->stream));
    st = build_layout(s, FEEC_METHOD_RAINBOW, Dd, omega, hR.data(), Fd, fptr, bptr, brows, num_colors);
    if (st == FEEC_OK) {
        // each color's rows are longest first: where its long rows end, in both sweeps' order
        std::vector<int> fsplit((size_t)num_colors), bsplit((size_t)num_colors);
        for (int c = 0; c < num_colors; c++) {
            int k = hB[c];
            while (k < hB[c + 1] && hA[hR[k] + 1] - hA[hR[k]] > kLongRowEntries) k++;
            fsplit[c] = k;
            const int p = num_colors - 1 - c;   // backward phase of color c: slots bptr[p].. hold rows hB[c]..
            bsplit[p] = bptr[p] + (k - hB[c]);
        }
        DevArena& M = s->mem;
        FEEC_TRY(M.alloc(s->fsplit, fsplit.size() + 1));
        FEEC_TRY(M.alloc(s->bsplit, bsplit.size() + 1));
        FEEC_TRY(cudaMemcpyAsync(s->fsplit, fsplit.data(), sizeof(int) * fsplit.size(), cudaMemcpyHostToDevice, s->stream));
        FEEC_TRY(cudaMemcpyAsync(s->bsplit, bsplit.data(), sizeof(int) * bsplit.size(), cudaMemcpyHostToDevice, s->stream));
    }
    tmp.release();
    cudaStreamSynchronize(s->stream);
    return st;
}

int feec_system_set_diagonal_precon(feec_system* s, const double* precon, int host_ptrs) {
    if (!s || !precon) return FEEC_BADARG;
    if (!s->precon) {
        HomeStreamScope home(s);
        FEEC_TRY(s->mem.alloc(s->precon, (size_t)s->n));
    }
    FEEC_TRY(cudaMemcpyAsync(s->precon, precon, sizeof(double) * s->n,
                             host_ptrs ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s->stream));
    FEEC_TRY(cudaStreamSynchronize(s->stream));
    return FEEC_OK;
}

int feec_system_set_ssor(feec_system* s, const double* diagonal, double omega, int host_ptrs) {
    if (!s || !diagonal || !(omega > 0.0) || !(omega < 2.0)) return FEEC_BADARG;
    const int n = s->n;
    std::vector<int> hA, hC;
    int st = FEEC_OK;
    // the level computation needs the pattern on the host
    hA.resize((size_t)n + 1); hC.resize((size_t)s->nnz);
    FEEC_TRY(cudaMemcpyAsync(hA.data(), s->A, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s->stream));
    FEEC_TRY(cudaMemcpyAsync(hC.data(), s->C, sizeof(int) * (size_t)s->nnz, cudaMemcpyDeviceToHost, s->stream));
    FEEC_TRY(cudaStreamSynchronize(s->stream));
    std::vector<int> flev, blev;
    int nfl = 0, nbl = 0;
    triangular_levels(n, hA.data(), hC.data(), true, flev, nfl);
    triangular_levels(n, hA.data(), hC.data(), false, blev, nbl);
    // rows renumbered by forward level (stable), backward schedule listed in the new numbering
    std::vector<int> fcount((size_t)nfl + 1, 0), perm((size_t)n), iperm((size_t)n);
    for (int i = 0; i < n; i++) fcount[flev[i] + 1]++;
    for (int l = 0; l < nfl; l++) fcount[l + 1] += fcount[l];
    std::vector<int> fptr(fcount.begin(), fcount.end());
    for (int i = 0; i < n; i++) { const int p = fcount[flev[i]]++; perm[p] = i; iperm[i] = p; }
    std::vector<int> bcount((size_t)nbl + 1, 0), brows((size_t)n);
    for (int i = 0; i < n; i++) bcount[blev[i] + 1]++;
    for (int l = 0; l < nbl; l++) bcount[l + 1] += bcount[l];
    std::vector<int> bptr(bcount.begin(), bcount.end());
    for (int i = n - 1; i >= 0; i--) brows[bcount[blev[i]]++] = iperm[i];
    DevArena tmp; tmp.stream = s->stream;
    double* Dd = nullptr;
    FEEC_TRY(tmp.alloc(Dd, n));
    FEEC_TRY(cudaMemcpyAsync(Dd, diagonal, sizeof(double) * n, host_ptrs ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s->stream));
    st = build_layout(s, FEEC_METHOD_SSOR, Dd, omega, perm.data(), nullptr, fptr, bptr, brows, nfl);
    tmp.release();
    cudaStreamSynchronize(s->stream);
    return st;
}

int feec_system_solve(feec_system* s, int method, int mode, double* x, const double* b, double* residual,
                      double precision, int max_iter, feec_solve_info* info, void* stream) {
    zero_info(info);
    if (!s || !x || !b || !(precision > 0.0)) return FEEC_BADARG;
    if (method < FEEC_METHOD_CG || method > FEEC_METHOD_DIAGONAL || mode < FEEC_MODE_REFERENCE || mode > FEEC_MODE_MIXED)
        return FEEC_BADARG;
    cudaStream_t keep = s->stream;
    if (stream) s->stream = (cudaStream_t)stream;
    const auto t0 = std::chrono::steady_clock::now();
    int st = solve_core(s, method, mode, x, b, residual, precision, max_iter, 0.0, -3, info);
    if (info) info->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    s->stream = keep;
    return st;
}

int feec_system_apply(feec_system* s, const double* x, double* y, double scaling, void* stream) {
    if (!s || !x || !y) return FEEC_BADARG;
    cudaStream_t keep = s->stream;
    if (stream) s->stream = (cudaStream_t)stream;
    int e = FEEC_OK;
    if (s->user_lanes > 0) {
        // launch-shape override: the CSR kernel with the requested lanes per row
        e = cuda_status(launch_spmv_f64(s->n, s->A, s->C, s->V, x, y, scaling, s->user_lanes, s->stream));
    } else {
        e = sell_prepare(s, FEEC_METHOD_CG);
        if (e == FEEC_OK) {
            const SellView v = sell_view(s, FEEC_METHOD_CG);
            e = cuda_status(launch_sell_spmv(v, 0, x, y, scaling, s->stream));
        }
    }
    s->stream = keep;
    return e;
}

int feec_system_apply_f32(feec_system* s, const float* x, float* y, float scaling, void* stream) {
    if (!s || !x || !y) return FEEC_BADARG;
    cudaStream_t keep = s->stream;
    if (stream) s->stream = (cudaStream_t)stream;
    int e = sell_prepare(s, FEEC_METHOD_CG);
    if (e == FEEC_OK) {
        const SellView v = sell_view(s, FEEC_METHOD_CG);
        e = cuda_status(launch_sell_spmv(v, 1, x, y, (double)scaling, s->stream));
    }
    s->stream = keep;
    return e;
}

// ---------------------------------------------------------------------------
// Drop-in host-pointer entry points
// ---------------------------------------------------------------------------

static int dropin_solve(int method, int N, double* x, const double* b, const int* A, const int* C, const double* V,
                        double* residual, double precision, int print_modulo, const double* diagonal, double omega,
                        int num_colors, const int* F, const int* B, const int* R, feec_solve_info* info) {
    zero_info(info);
    // the reference asserts these (sparsesolver.cpp:32-43, 1013-1027)
    if (N <= 0 || !x || !b || !A || !C || !V || !residual || !(precision > 0.0)) return FEEC_BADARG;
    const bool rb = method == FEEC_METHOD_RAINBOW || method == FEEC_METHOD_RAINBOW_EISENSTAT;
    if (method != FEEC_METHOD_CG && !diagonal) return FEEC_BADARG;
    if (rb && (num_colors < 0 || !F || !B || !R)) return FEEC_BADARG;
    const auto t0 = std::chrono::steady_clock::now();
    const double tolerance = host_tolerance(N, b, precision);
    if (print_modulo >= -1) std::printf("(%d/%d)     BEGIN: %s\n", 0, N, method_title(method));

    feec_system* s = nullptr;
    int st = feec_system_create(&s, N, A, C, V, 1, nullptr);
    if (st != FEEC_OK) return st;
    if (rb) st = feec_system_set_rainbow(s, diagonal, omega, num_colors, F, B, R, 1);
    else if (method == FEEC_METHOD_DIAGONAL) st = feec_system_set_diagonal_precon(s, diagonal, 1);
    else if (method != FEEC_METHOD_CG) st = feec_system_set_ssor(s, diagonal, omega, 1);
    double *dx = nullptr, *db = nullptr, *dr = nullptr;
    DevArena io; io.stream = s->stream;
    if (st == FEEC_OK) {
        cudaError_t e;
        if ((e = io.alloc(dx, N)) != cudaSuccess || (e = io.alloc(db, N)) != cudaSuccess || (e = io.alloc(dr, N)) != cudaSuccess ||
            (e = cudaMemcpyAsync(dx, x, sizeof(double) * N, cudaMemcpyHostToDevice, s->stream)) != cudaSuccess ||
            (e = cudaMemcpyAsync(db, b, sizeof(double) * N, cudaMemcpyHostToDevice, s->stream)) != cudaSuccess ||
            (e = cudaMemcpyAsync(dr, residual, sizeof(double) * N, cudaMemcpyHostToDevice, s->stream)) != cudaSuccess)
            st = cuda_status(e);
    }
    feec_solve_info local;
    feec_solve_info* inf = info ? info : &local;
    zero_info(inf);
    if (st == FEEC_OK) st = solve_core(s, method, FEEC_MODE_REFERENCE, dx, db, dr, precision, N, tolerance, print_modulo, inf);
    const bool solved = st == FEEC_OK || st == FEEC_BREAKDOWN || st == FEEC_SMALL_ENERGY || st == FEEC_MAXITER;
    if (solved) {
        cudaError_t e = cudaMemcpyAsync(x, dx, sizeof(double) * N, cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(residual, dr, sizeof(double) * N, cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) st = cuda_status(e);
    }
    io.release();
    feec_system_destroy(s);
    inf->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    inf->tolerance = tolerance;
    if (solved && print_modulo >= -2) {
        if (st == FEEC_BREAKDOWN)
            std::printf("(%d/%d) BREAKDOWN: Gradient energy is unreasonable\n", inf->iterations, N);
        else if (st == FEEC_SMALL_ENERGY)
            std::printf("(%d/%d)   WARNING: Gradient energy is small\n", inf->iterations, N);
    }
    if (solved && print_modulo >= -1)
        std::printf("(%d/%d) %9s: Residual norm is %.9le < %.9le\n", inf->iterations, N,
                    inf->final_norm < tolerance ? "SUCCESS" : "FAILED", inf->final_norm, tolerance);
    return st;
}

int feec_cg_csr(int N, double* x, const double* b, const int* A, const int* C, const double* V, double* residual,
                double precision, int print_modulo, feec_solve_info* info) {
    return dropin_solve(FEEC_METHOD_CG, N, x, b, A, C, V, residual, precision, print_modulo, nullptr, 1.0, 0, nullptr,
                        nullptr, nullptr, info);
}

int feec_cg_csr_ssor(int N, double* x, const double* b, const int* A, const int* C, const double* V, double* residual,
                     double precision, int print_modulo, const double* diagonal, double omega, feec_solve_info* info) {
    return dropin_solve(FEEC_METHOD_SSOR, N, x, b, A, C, V, residual, precision, print_modulo, diagonal, omega, 0,
                        nullptr, nullptr, nullptr, info);
}

int feec_cg_csr_rainbow(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                        double* residual, double precision, int print_modulo, const double* diagonal, double omega,
                        int num_colors, const int* F, const int* B, const int* R, feec_solve_info* info) {
    return dropin_solve(FEEC_METHOD_RAINBOW, N, x, b, A, C, V, residual, precision, print_modulo, diagonal, omega,
                        num_colors, F, B, R, info);
}

int feec_cg_csr_diagonal_precon(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                                double* residual, double precision, int print_modulo, const double* precon,
                                feec_solve_info* info) {
    return dropin_solve(FEEC_METHOD_DIAGONAL, N, x, b, A, C, V, residual, precision, print_modulo, precon, 1.0, 0,
                        nullptr, nullptr, nullptr, info);
}

int feec_cg_csr_ssor_eisenstat(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                               double* residual, double precision, int print_modulo, const double* diagonal,
                               double omega, feec_solve_info* info) {
    return dropin_solve(FEEC_METHOD_SSOR_EISENSTAT, N, x, b, A, C, V, residual, precision, print_modulo, diagonal,
                        omega, 0, nullptr, nullptr, nullptr, info);
}

int feec_cg_csr_eisenstat_rainbow(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                                  double* residual, double precision, int print_modulo, const double* diagonal,
                                  double omega, int num_colors, const int* F, const int* B, const int* R,
                                  feec_solve_info* info) {
    return dropin_solve(FEEC_METHOD_RAINBOW_EISENSTAT, N, x, b, A, C, V, residual, precision, print_modulo, diagonal,
                        omega, num_colors, F, B, R, info);
}

int feec_csr_apply(int rows, int cols, const int* A, const int* C, const double* V, const double* src, double* dest,
                   double scaling) {
    if (rows < 0 || cols < 0 || !A || (rows > 0 && (!dest)) || (cols > 0 && !src)) return FEEC_BADARG;
    if (rows == 0) return FEEC_OK;
    const int nnz = A[rows];
    if (nnz < 0 || (nnz > 0 && (!C || !V))) return FEEC_BADARG;
    int dev = 0;
    cudaStream_t s = nullptr;
    int st = init_device(dev, s);
    if (st != FEEC_OK) return st;
    DevArena m; m.stream = s;
    int *dA = nullptr, *dC = nullptr, *bad = nullptr; double *dV = nullptr, *dx = nullptr, *dy = nullptr;
    int bad_h = 0;
    cudaError_t e;
    // the matrix is checked on the device before the SpMV indexes through it
    if ((e = m.alloc(dA, (size_t)rows + 1)) == cudaSuccess && (e = m.alloc(dC, (size_t)nnz)) == cudaSuccess &&
        (e = m.alloc(dV, (size_t)nnz)) == cudaSuccess && (e = m.alloc(dx, (size_t)cols)) == cudaSuccess &&
        (e = m.alloc(dy, (size_t)rows)) == cudaSuccess && (e = m.alloc(bad, 1)) == cudaSuccess &&
        (e = cudaMemsetAsync(bad, 0, sizeof(int), s)) == cudaSuccess &&
        (e = cudaMemcpyAsync(dA, A, sizeof(int) * ((size_t)rows + 1), cudaMemcpyHostToDevice, s)) == cudaSuccess &&
        (nnz == 0 || (e = cudaMemcpyAsync(dC, C, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, s)) == cudaSuccess) &&
        (e = launch_validate_csr_cols(rows, cols, nnz, dA, dC, bad, s)) == cudaSuccess &&
        (e = cudaMemcpyAsync(&bad_h, bad, sizeof(int), cudaMemcpyDeviceToHost, s)) == cudaSuccess &&
        (e = cudaStreamSynchronize(s)) == cudaSuccess && !bad_h &&
        (nnz == 0 || (e = cudaMemcpyAsync(dV, V, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, s)) == cudaSuccess) &&
        (cols == 0 || (e = cudaMemcpyAsync(dx, src, sizeof(double) * (size_t)cols, cudaMemcpyHostToDevice, s)) == cudaSuccess) &&
        (e = launch_spmv_f64(rows, dA, dC, dV, dx, dy, scaling, pick_lanes((double)nnz / rows), s)) == cudaSuccess &&
        (e = cudaMemcpyAsync(dest, dy, sizeof(double) * (size_t)rows, cudaMemcpyDeviceToHost, s)) == cudaSuccess) {
        e = cudaStreamSynchronize(s);
    }
    m.release();
    cudaStreamSynchronize(s);
    if (e == cudaSuccess && bad_h) return FEEC_BADARG;
    return cuda_status(e);
}

int feec_csr_diagonal(int N, const int* A, const int* C, const double* V, double* diagonal) {
    if (N < 0 || !A || !diagonal) return FEEC_BADARG;
    if (N == 0) return FEEC_OK;
    const int nnz = A[N];
    int dev = 0;
    cudaStream_t s = nullptr;
    int st = init_device(dev, s);
    if (st != FEEC_OK) return st;
    DevArena m; m.stream = s;
    int *dA = nullptr, *dC = nullptr; double *dV = nullptr, *dd = nullptr;
    cudaError_t e;
    if ((e = m.alloc(dA, (size_t)N + 1)) == cudaSuccess && (e = m.alloc(dC, (size_t)nnz)) == cudaSuccess &&
        (e = m.alloc(dV, (size_t)nnz)) == cudaSuccess && (e = m.alloc(dd, (size_t)N)) == cudaSuccess &&
        (e = cudaMemcpyAsync(dA, A, sizeof(int) * ((size_t)N + 1), cudaMemcpyHostToDevice, s)) == cudaSuccess &&
        (nnz == 0 || (e = cudaMemcpyAsync(dC, C, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, s)) == cudaSuccess) &&
        (nnz == 0 || (e = cudaMemcpyAsync(dV, V, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, s)) == cudaSuccess) &&
        (e = launch_diagonal_f64(N, dA, dC, dV, dd, s)) == cudaSuccess &&
        (e = cudaMemcpyAsync(diagonal, dd, sizeof(double) * (size_t)N, cudaMemcpyDeviceToHost, s)) == cudaSuccess) {
        e = cudaStreamSynchronize(s);
    }
    m.release();
    cudaStreamSynchronize(s);
    return cuda_status(e);
}

int feec_rainbow(int N, const int* A, const int* C, int* num_colors, int* F, int* B, int* R) {
    if (N < 0 || !A || !num_colors || (N > 0 && (!C || !F || !B || !R))) return FEEC_BADARG;
    if (N == 0) { *num_colors = 0; if (B) B[0] = 0; return FEEC_OK; }
    *num_colors = rainbow_host(N, A, C, F, B, R);
    return FEEC_OK;
}

int feec_csr_check(int rows, int cols, const int* A, const int* C, const double* V) {
    if (rows < 0 || cols < 0 || !A) return FEEC_BADARG;
    if (A[0] != 0) return FEEC_BADARG;
    for (int p = 1; p <= rows; p++) if (A[p - 1] > A[p]) return FEEC_BADARG;
    const int nnz = A[rows];
    for (int i = 0; i < nnz; i++)
        if (C[i] < 0 || C[i] >= cols || !std::isfinite(V[i])) return FEEC_BADARG;
    return FEEC_OK;
}

}  // extern "C"
