// The remaining CSR Krylov drivers of solver/sparsesolver.cpp, each one cooperative
// persistent launch per solve over the caller's CSR (FP64, the reference's stopping rules):
//
//   cr_persistent        — ConjugateResidualSolverCSR (:1687-1915) and its _textbook twin
//                          (:1918-2156; the same arithmetic, only names and messages differ)
//   minres_persistent    — MINRESCSR (:2159-2425)
//   chebyshev_persistent — ChebyshevIteration_DiagonalPreconditioner (:2428-2590)
//
// As in the CG kernels, every grid-wide sum is reduced deterministically (per-block
// partials, then every block adds them in the same order), scalar recurrences run in
// thread 0 of every block on identical inputs and are broadcast through shared memory,
// and consecutive reductions alternate between two partial arrays so that a block that
// runs ahead never overwrites partials another block is still adding.
//
// The reference restarts only at K = 0 (csr_restart_on_full_dimension and
// csr_restart_before_finish are false, :21-22), so each kernel starts once.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "persistent_common.cuh"
#include "feec_system.h"

namespace feec {
namespace {

struct MoreArgs {
    int n;
    const int* rp;
    const int* ci;
    const double* val;
    const double* b;
    double* x;
    double* res;
    double* w[7];            // work vectors (NaN on entry, as the reference allocates them)
    const double* precon;    // Chebyshev
    double lower, upper;     // Chebyshev spectral bounds
    double tol;              // max(precision * ||b||, 2^-26)
    int print_modulo;
    int max_iter;            // the reference's N
    double* partials;        // 4 * gridDim.x doubles
    DeviceStatus* st;
};

// ---------------------------------------------------------------------------
// Conjugate residuals
// ---------------------------------------------------------------------------
template <int LANES>
__global__ void __launch_bounds__(kThreads) cr_persistent(MoreArgs a) {
    unsigned long long epoch = 0;
    const int n = a.n;
    const int lane = threadIdx.x & (LANES - 1);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nthr = gridDim.x * blockDim.x;
    double* pA = a.partials;
    double* pB = a.partials + 2 * gridDim.x;
    double* dir = a.w[0];
    double* Adir = a.w[1];
    double* Ares = a.w[2];
    double* vil = a.w[3];

    // restart (:1749-1790): res = b - A x, dir = res; then Adir = A dir, Ares = Adir
    FEEC_FOR_ROW_GROUPS(0, n, i, act) {
        const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
        const double s = seg_dot<double, LANES>(a.ci, a.val, a.x, lo, hi, lane);
        if (act && lane == 0) {
            const double r = __ldg(&a.b[i]) - s;
            a.res[i] = r;
            dir[i] = r;
        }
    }
    if (!grid_barrier(a.st, epoch, 40)) return;
    double adr = 0.0, adad = 0.0;
    FEEC_FOR_ROW_GROUPS(0, n, i, act) {
        const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
        const double s = seg_dot<double, LANES>(a.ci, a.val, dir, lo, hi, lane);
        if (act && lane == 0) {
            Adir[i] = s;
            Ares[i] = s;
            adr += s * a.res[i];
            adad += s * s;
        }
    }
    write_partials2<double>(pA, adr, adad);
    if (!grid_barrier(a.st, epoch, 41)) return;
    double v2[2];
    grid_sum<2>(pA, v2);
    double Ad_r = v2[0], Ad_Ad = v2[1];

    __shared__ double s_scal;
    __shared__ int s_ctl;
    int K = 0;
    int status = FEEC_MAXITER;
    while (K < a.max_iter) {
        if (threadIdx.x == 0) {
            if (a.print_modulo > 0 && K % a.print_modulo == 0 && blockIdx.x == 0)
                printf("(%d/%d)   INTERIM: Residual norm is %.9le < %.9le\n", K, n, sqrt(Ad_r), a.tol);
            int ctl = 0;
            if (!isfinite(Ad_r) || Ad_r < 0.0) ctl = 1;                                // :1804-1809
            else if (fabs(Ad_r) < a.tol * a.tol) ctl = 3;                              // :1811-1812
            else if (!isfinite(Ad_Ad) || Ad_Ad < 0.0) ctl = 1;                         // :1819-1824
            else if (sqrt(fabs(Ad_Ad)) < kMachineEpsilon) ctl = 2;                     // :1826-1830
            s_ctl = ctl;
            s_scal = Ad_r / Ad_Ad;                                                     // :1840
        }
        __syncthreads();
        if (s_ctl == 3) { status = FEEC_OK; break; }
        if (s_ctl == 1) { status = FEEC_BREAKDOWN; break; }
        if (s_ctl == 2) { status = FEEC_SMALL_ENERGY; break; }
        const double alpha = s_scal;

        // :1846-1863: vil = A Adir; x, res, Ares updated; Ares.res
        double acc = 0.0;
        FEEC_FOR_ROW_GROUPS(0, n, i, act) {
            const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
            const double s = seg_dot<double, LANES>(a.ci, a.val, Adir, lo, hi, lane);
            if (act && lane == 0) {
                vil[i] = s;
                a.x[i] = a.x[i] + alpha * dir[i];
                const double r = a.res[i] - alpha * Adir[i];
                a.res[i] = r;
                const double ar = Ares[i] - alpha * s;
                Ares[i] = ar;
                acc += ar * r;
            }
        }
        write_partials<double>(pB, acc);
        if (!grid_barrier(a.st, epoch, 42)) return;
        double v1[1];
        grid_sum<1>(pB, v1);
        const double new_Ar_r = v1[0];
        if (threadIdx.x == 0) s_scal = new_Ar_r / Ad_r;                                 // :1865
        __syncthreads();
        const double beta = s_scal;

        // :1867-1880: dir, Adir and Adir.Adir
        double aa = 0.0;
        for (int i = tid; i < n; i += nthr) {
            dir[i] = a.res[i] + beta * dir[i];
            const double ad = Ares[i] + beta * Adir[i];
            Adir[i] = ad;
            aa += ad * ad;
        }
        write_partials<double>(pA, aa);
        if (!grid_barrier(a.st, epoch, 43)) return;
        grid_sum<1>(pA, v1);
        Ad_Ad = v1[0];
        Ad_r = new_Ar_r;
        K++;
    }
    finish(a.st, status, K, Ad_r, Ad_Ad);
}

// ---------------------------------------------------------------------------
// MINRES
// ---------------------------------------------------------------------------
template <int LANES>
__global__ void __launch_bounds__(kThreads) minres_persistent(MoreArgs a) {
    unsigned long long epoch = 0;
    const int n = a.n;
    const int lane = threadIdx.x & (LANES - 1);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nthr = gridDim.x * blockDim.x;
    double* pA = a.partials;
    double* pB = a.partials + 2 * gridDim.x;
    double* v0 = a.w[0];
    double* v1 = a.w[1];
    double* w0 = a.w[2];
    double* w1 = a.w[3];
    double* vn = a.w[4];
    double* wn = a.w[5];
    double* p = a.w[6];

    // restart (:2233-2283): v0 = w0 = w1 = 0, v1 = (b - A x) / gamma
    double acc = 0.0;
    FEEC_FOR_ROW_GROUPS(0, n, i, act) {
        const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
        const double s = seg_dot<double, LANES>(a.ci, a.val, a.x, lo, hi, lane);
        if (act && lane == 0) {
            v0[i] = 0.0; w0[i] = 0.0; w1[i] = 0.0;
            const double r = __ldg(&a.b[i]) - s;
            v1[i] = r;
            acc += r * r;
        }
    }
    write_partials<double>(pA, acc);
    if (!grid_barrier(a.st, epoch, 50)) return;
    double v[1];
    grid_sum<1>(pA, v);
    double gamma = sqrt(v[0]);
    for (int i = tid; i < n; i += nthr) v1[i] /= gamma;
    if (!grid_barrier(a.st, epoch, 51)) return;

    // scalar state, kept by thread 0 of every block (identical inputs in every block)
    double s0 = 0.0, s1 = 0.0, c0 = 1.0, c1 = 1.0, eta = gamma;
    __shared__ double s_sc[5];
    __shared__ int s_ctl;
    int K = 0;
    int status = FEEC_MAXITER;
    while (K < a.max_iter) {
        if (threadIdx.x == 0) s_ctl = fabs(eta) < a.tol ? 1 : 0;                       // :2290-2293
        __syncthreads();
        if (s_ctl) { status = FEEC_OK; break; }

        // :2297-2313: p = A v1, delta = p.v1
        acc = 0.0;
        FEEC_FOR_ROW_GROUPS(0, n, i, act) {
            const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
            const double s = seg_dot<double, LANES>(a.ci, a.val, v1, lo, hi, lane);
            if (act && lane == 0) {
                p[i] = s;
                acc += s * v1[i];
            }
        }
        write_partials<double>(pB, acc);
        if (!grid_barrier(a.st, epoch, 52)) return;
        grid_sum<1>(pB, v);
        const double delta = v[0];

        // :2317-2330: vn = p - delta v1 - gamma v0, gamma_n^2 = vn.vn
        acc = 0.0;
        for (int i = tid; i < n; i += nthr) {
            const double t = p[i] - delta * v1[i] - gamma * v0[i];
            vn[i] = t;
            acc += t * t;
        }
        write_partials<double>(pA, acc);
        if (!grid_barrier(a.st, epoch, 53)) return;
        grid_sum<1>(pA, v);
        const double gamma_n = sqrt(v[0]);
        if (threadIdx.x == 0) {                                                        // :2338-2349
            const double alpha_0 = c1 * delta - c0 * s1 * gamma;
            const double alpha_1 = sqrt(alpha_0 * alpha_0 + gamma_n * gamma_n);
            const double alpha_2 = s1 * delta + c0 * c1 * gamma;
            const double alpha_3 = s0 * gamma;
            const double cn = alpha_0 / alpha_1;
            const double sn = gamma_n / alpha_1;
            s_sc[0] = alpha_1; s_sc[1] = alpha_2; s_sc[2] = alpha_3; s_sc[3] = cn * eta;
            eta = -sn * eta;                                                           // :2362
            c0 = c1; s0 = s1; c1 = cn; s1 = sn;
        }
        __syncthreads();
        const double alpha_1 = s_sc[0], alpha_2 = s_sc[1], alpha_3 = s_sc[2], ce = s_sc[3];
        // :2332-2360: vn normalised; wn = (v1 - alpha_2 w1 - alpha_3 w0) / alpha_1; x += cn eta wn
        for (int i = tid; i < n; i += nthr) {
            vn[i] /= gamma_n;
            const double t = (v1[i] - alpha_2 * w1[i] - alpha_3 * w0[i]) / alpha_1;
            wn[i] = t;
            a.x[i] = a.x[i] + ce * t;
        }
        if (!grid_barrier(a.st, epoch, 54)) return;
        // :2364-2378: v0 <- v1 <- vn, w0 <- w1 <- wn (the freed vectors become vn, wn)
        double* t = v0; v0 = v1; v1 = vn; vn = t;
        t = w0; w0 = w1; w1 = wn; wn = t;
        gamma = gamma_n;
        if (threadIdx.x == 0 && blockIdx.x == 0 && a.print_modulo > 0 && K % a.print_modulo == 0)
            printf("(%d/%d)   INTERIM: Residual norm is %.9le < %.9le\n", K, n, eta, a.tol);
        K++;
    }
    // :2397-2403: res = b - A x
    FEEC_FOR_ROW_GROUPS(0, n, i, act) {
        const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
        const double s = seg_dot<double, LANES>(a.ci, a.val, a.x, lo, hi, lane);
        if (act && lane == 0) a.res[i] = __ldg(&a.b[i]) - s;
    }
    if (threadIdx.x == 0) s_sc[4] = eta;
    __syncthreads();
    finish(a.st, status, K, s_sc[4], gamma);
}

// ---------------------------------------------------------------------------
// Chebyshev iteration with a diagonal preconditioner
// ---------------------------------------------------------------------------
template <int LANES>
__global__ void __launch_bounds__(kThreads) chebyshev_persistent(MoreArgs a) {
    unsigned long long epoch = 0;
    const int n = a.n;
    const int lane = threadIdx.x & (LANES - 1);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nthr = gridDim.x * blockDim.x;
    double* part[2] = {a.partials, a.partials + 2 * gridDim.x};
    double* xp = a.w[0];
    double* xc = a.w[1];
    double* xn = a.w[2];
    const double alpha = 2. / (a.upper + a.lower);                                    // :2486-2487
    const double mu = (a.upper + a.lower) / (a.upper - a.lower);

    // :2476-2480 and the restart :2499-2531 (x_prev = x): residual, x_curr = x_prev + alpha z.
    // The product reads x itself, which holds the same values as x_prev.
    double acc = 0.0;
    FEEC_FOR_ROW_GROUPS(0, n, i, act) {
        const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
        const double s = seg_dot<double, LANES>(a.ci, a.val, a.x, lo, hi, lane);
        if (act && lane == 0) {
            const double xi = a.x[i];
            xp[i] = xi; xn[i] = xi;
            const double r = __ldg(&a.b[i]) - s;
            a.res[i] = r;
            const double z = __ldg(&a.precon[i]) * r;
            xc[i] = xi + alpha * z;
            acc += r * r;
        }
    }
    write_partials<double>(part[0], acc);
    if (!grid_barrier(a.st, epoch, 60)) return;
    double v[1];
    grid_sum<1>(part[0], v);
    double r_r = v[0];
    double gamma_prev = 1., gamma_curr = mu;

    __shared__ double s_om;
    __shared__ int s_ctl;
    int K = 0;
    int status = FEEC_MAXITER;
    while (K < a.max_iter) {
        if (threadIdx.x == 0) {
            s_ctl = sqrt(r_r) < a.tol ? 1 : 0;                                          // :2535-2538
            const double gamma_next = 2. * mu * gamma_curr - gamma_prev;               // :2542
            s_om = 2. * mu * gamma_curr / gamma_next;                                  // :2543
            gamma_prev = gamma_curr;
            gamma_curr = gamma_next;
        }
        __syncthreads();
        if (s_ctl) { status = FEEC_OK; break; }
        const double omega = s_om;
        // :2545-2563: residual of x_curr, x_next = x_prev + omega (alpha z + x_curr - x_prev)
        acc = 0.0;
        FEEC_FOR_ROW_GROUPS(0, n, i, act) {
            const int lo = act ? __ldg(&a.rp[i]) : 0, hi = act ? __ldg(&a.rp[i + 1]) : 0;
            const double s = seg_dot<double, LANES>(a.ci, a.val, xc, lo, hi, lane);
            if (act && lane == 0) {
                const double r = __ldg(&a.b[i]) - s;
                a.res[i] = r;
                const double z = __ldg(&a.precon[i]) * r;
                xn[i] = xp[i] + omega * (alpha * z + xc[i] - xp[i]);
                acc += r * r;
            }
        }
        double* pk = part[(K + 1) & 1];
        write_partials<double>(pk, acc);
        if (!grid_barrier(a.st, epoch, 61)) return;
        grid_sum<1>(pk, v);
        r_r = v[0];
        // :2568-2569: x_prev <- x_curr, x_curr <- x_next, x_next <- the old x_prev
        double* t = xp; xp = xc; xc = xn; xn = t;
        if (threadIdx.x == 0 && blockIdx.x == 0 && a.print_modulo > 0 && K % a.print_modulo == 0)
            printf("(%d/%d)   INTERIM: Residual norm is %.9le < %.9le\n", K, n, sqrt(r_r), a.tol);
        K++;
    }
    for (int i = tid; i < n; i += nthr) a.x[i] = xn[i];                                 // :2578-2582
    finish(a.st, status, K, r_r, 0.0);
}

enum { kKindCR = 0, kKindCRTextbook = 1, kKindMinres = 2, kKindChebyshev = 3 };

template <int LANES>
const void* more_fn(int kind) {
    if (kind == kKindMinres) return (const void*)minres_persistent<LANES>;
    if (kind == kKindChebyshev) return (const void*)chebyshev_persistent<LANES>;
    return (const void*)cr_persistent<LANES>;
}

const void* more_kernel(int kind, int lanes) {
    switch (lanes) {
        case 1: return more_fn<1>(kind);
        case 4: return more_fn<4>(kind);
        default: return more_fn<8>(kind);
    }
}

const char* more_title(int kind) {
    switch (kind) {
        case kKindCR: return "Conjugate Residual CSR";
        case kKindCRTextbook: return "Conjugate Residual CSR (textbook)";
        case kKindMinres: return "MINRES CSR";
        default: return "Chebyshev (Diag) CSR";
    }
}

void clear_info(feec_solve_info* info) {
    if (!info) return;
    std::memset(info, 0, sizeof(*info));
    info->true_relres = -1.0;
    info->outer_iterations = 1;
    info->error_estimate = -1.0;
}

int more_dropin(int kind, int N, double* x, const double* b, const int* A, const int* C, const double* V,
                double* residual, double precision, int print_modulo, const double* precon, double lower,
                double upper, feec_solve_info* info) {
    clear_info(info);
    // the reference asserts these (:1699-1706, :2171-2178, :2441-2449)
    if (N <= 0 || !x || !b || !A || !C || !V || !residual || !(precision > 0.0)) return FEEC_BADARG;
    if (kind == kKindChebyshev && !precon) return FEEC_BADARG;
    const auto t0 = std::chrono::steady_clock::now();
    double tolerance = 0.0;                                   // serial, as the reference
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = precision * std::sqrt(tolerance);
    tolerance = std::max(tolerance, 1.490116119384765625e-08);
    const int nnz = A[N];
    if (nnz < 0) return FEEC_BADARG;
    if (kind == kKindChebyshev) std::printf("%g %g\n", lower, upper);                   // :2484
    if (print_modulo >= -1) std::printf("(%d/%d)     BEGIN: %s\n", 0, N, more_title(kind));

    int dev = 0;
    cudaStream_t s = nullptr;
    int st = init_device(dev, s);
    if (st != FEEC_OK) return st;
    DevArena m;
    m.stream = s;
    struct Release { DevArena& m; cudaStream_t s; ~Release() { m.release(); cudaStreamSynchronize(s); } } rel{m, s};
    int *dA, *dC, *bad; double *dV, *db, *dx, *dres, *dpre = nullptr, *part; DeviceStatus* dst;
    double* w[7] = {};
    FEEC_TRY(m.alloc(dA, (size_t)N + 1)); FEEC_TRY(m.alloc(dC, (size_t)std::max(nnz, 1)));
    FEEC_TRY(m.alloc(dV, (size_t)std::max(nnz, 1))); FEEC_TRY(m.alloc(bad, 1));
    FEEC_TRY(m.alloc(db, (size_t)N)); FEEC_TRY(m.alloc(dx, (size_t)N)); FEEC_TRY(m.alloc(dres, (size_t)N));
    for (int k = 0; k < 7; k++) FEEC_TRY(m.alloc(w[k], (size_t)N));
    if (kind == kKindChebyshev) FEEC_TRY(m.alloc(dpre, (size_t)N));
    FEEC_TRY(m.alloc(dst, 1));
    FEEC_TRY(cudaMemcpyAsync(dA, A, sizeof(int) * ((size_t)N + 1), cudaMemcpyHostToDevice, s));
    if (nnz > 0) {
        FEEC_TRY(cudaMemcpyAsync(dC, C, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, s));
        FEEC_TRY(cudaMemcpyAsync(dV, V, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, s));
    }
    FEEC_TRY(cudaMemcpyAsync(db, b, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, s));
    FEEC_TRY(cudaMemcpyAsync(dx, x, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, s));
    FEEC_TRY(cudaMemcpyAsync(dres, residual, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, s));
    if (dpre) FEEC_TRY(cudaMemcpyAsync(dpre, precon, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, s));
    for (int k = 0; k < 7; k++) FEEC_TRY(cudaMemsetAsync(w[k], 0xFF, sizeof(double) * (size_t)N, s));   // NaN
    FEEC_TRY(cudaMemsetAsync(bad, 0, sizeof(int), s));
    FEEC_TRY(cudaMemsetAsync(dst, 0, sizeof(DeviceStatus), s));
    // the kernels index x through C: the CSR is checked on the device first
    FEEC_TRY(launch_validate_csr(N, nnz, dA, dC, bad, s));
    int hbad = 0;
    FEEC_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));
    if (hbad) return FEEC_BADARG;

    // one thread per row for short rows (FP64 issue bound), lanes for long ones
    const double avg = (double)nnz / N;
    const int lanes = avg <= 32.0 ? 1 : (avg <= 96.0 ? 4 : 8);
    const void* fn = more_kernel(kind, lanes);
    int sms = 0, per_sm = 0;
    FEEC_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    FEEC_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, 0));
    const long long want = ((long long)N * lanes + kThreads - 1) / kThreads;
    int blocks = (int)std::min<long long>(want, (long long)std::min(per_sm, 2) * sms);
    if (blocks < 1) return FEEC_CUDA_ERROR;
    FEEC_TRY(m.alloc(part, (size_t)4 * blocks));

    MoreArgs args{};
    args.n = N; args.rp = dA; args.ci = dC; args.val = dV; args.b = db; args.x = dx; args.res = dres;
    for (int k = 0; k < 7; k++) args.w[k] = w[k];
    args.precon = dpre; args.lower = lower; args.upper = upper;
    args.tol = tolerance; args.print_modulo = print_modulo; args.max_iter = N;
    args.partials = part; args.st = dst;
    cudaEvent_t e0, e1;
    FEEC_TRY(cudaEventCreate(&e0)); FEEC_TRY(cudaEventCreate(&e1));
    void* params[] = {&args};
    cudaEventRecord(e0, s);
    note_launch();
    cudaError_t le = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(kThreads), params, 0, s);
    cudaEventRecord(e1, s);
    DeviceStatus hs{};
    if (le == cudaSuccess) le = cudaMemcpyAsync(&hs, dst, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s);
    if (le == cudaSuccess) le = cudaStreamSynchronize(s);
    float ms = 0.0f;
    if (le == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    if (le != cudaSuccess) return cuda_status(le);
    if (hs.status == FEEC_TIMEOUT) return FEEC_TIMEOUT;
    FEEC_TRY(cudaMemcpyAsync(x, dx, sizeof(double) * (size_t)N, cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaMemcpyAsync(residual, dres, sizeof(double) * (size_t)N, cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));

    // the norm each driver prints: sqrt(Ar.r) (CR; NaN for a negative energy, as printed by the
    // reference), eta (MINRES), sqrt(r.r) (Chebyshev); info gets the magnitude the rule tests
    const double shown = kind == kKindMinres ? hs.final_value : std::sqrt(hs.final_value);
    const double tested = kind == kKindMinres ? std::fabs(hs.final_value) : std::sqrt(std::fabs(hs.final_value));
    if (info) {
        info->status = hs.status;
        info->iterations = hs.iterations;
        info->tolerance = tolerance;
        info->final_norm = tested;
        info->device_ms = ms;
        info->grid_blocks = blocks;
        info->lanes_per_row = lanes;
        info->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    if (print_modulo >= -2 && (kind == kKindCR || kind == kKindCRTextbook)) {
        if (hs.status == FEEC_BREAKDOWN)
            std::printf("(%d/%d) BREAKDOWN: Residual or gradient energy is unreasonable with %.9le / %.9le\n",
                        hs.iterations, N, hs.final_value, hs.aux_value);
        else if (hs.status == FEEC_SMALL_ENERGY)
            std::printf("(%d/%d)   WARNING: Gradient double energy is small with %.9le\n", hs.iterations, N,
                        hs.aux_value);
    }
    if (print_modulo >= -1)
        std::printf("(%d/%d) %9s: Residual norm is %.9le < %.9le\n", hs.iterations, N,
                    shown < tolerance ? "SUCCESS" : "FAILED", shown, tolerance);
    return hs.status;
}

}  // namespace
}  // namespace feec

using namespace feec;

extern "C" {

int feec_cr_csr(int N, double* x, const double* b, const int* A, const int* C, const double* V, double* residual,
                double precision, int print_modulo, feec_solve_info* info) {
    return more_dropin(kKindCR, N, x, b, A, C, V, residual, precision, print_modulo, nullptr, 0.0, 0.0, info);
}

int feec_cr_csr_textbook(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                         double* residual, double precision, int print_modulo, feec_solve_info* info) {
    return more_dropin(kKindCRTextbook, N, x, b, A, C, V, residual, precision, print_modulo, nullptr, 0.0, 0.0,
                       info);
}

int feec_minres_csr(int N, double* x, const double* b, const int* A, const int* C, const double* V, double* residual,
                    double precision, int print_modulo, feec_solve_info* info) {
    return more_dropin(kKindMinres, N, x, b, A, C, V, residual, precision, print_modulo, nullptr, 0.0, 0.0, info);
}

int feec_chebyshev_diag(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                        double* residual, double precision, int print_modulo, const double* precon, double lower,
                        double upper, feec_solve_info* info) {
    return more_dropin(kKindChebyshev, N, x, b, A, C, V, residual, precision, print_modulo, precon, lower, upper,
                       info);
}

}  // extern "C"
