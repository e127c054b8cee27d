// Hodge conjugate residual solvers (solver/systemsparsesolver.cpp:18-1120) on the GPU:
// conjugate residuals on the Schur complement M = B A^-1 Bt + C of a mixed Hodge-Laplace
// system (A: L x L, B: N x L, Bt: L x N, C: N x N), A^-1 applied by an inner CG on A to
// inner_precision:
//
//   variant 0  HodgeConjugateResidualSolverCSR_diagonal  inner CG with precon 1/diag(A) (:52-424)
//   variant 1  HodgeConjugateResidualSolverCSR_SSOR      inner SSOR-PCG, omega = 1     (:426-796)
//              (and HodgeConjugateResidualSolverCSR, which forwards to it, :18-50)
//   variant 2  HodgeConjugateResidualSolverCSR_textbook  inner plain CG               (:798-1120)
//
// A stays resident as a feec_system; each inner solve is one persistent solve of the
// corresponding engine with the reference's stopping rule, on the system's stream, and the
// outer iteration's products with B, Bt and C and its vector updates are fused row kernels
// on the same stream. As in the reference, the inner solves of the restart start from zero
// and those of the iterations from the previous inner solution (:253-277). The outer
// scalars (two sums per iteration) come back to the host, which runs the outer control.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <vector>

#include "feec_internal.h"
#include "feec_system.h"

namespace feec {
namespace {

constexpr int kHBlock = 256;
constexpr double kSignA = 1.;                              // systemsparsesolver.hpp:8
constexpr double kEpsilon = 2.220446049250313080847263336181640625e-16;
constexpr double kDesired = 1.490116119384765625e-08;

int hgrid(int n, int cap) { return std::max(1, std::min(cap, (n + kHBlock - 1) / kHBlock)); }

// Block partial sums in a fixed order: thread sums, then a shared-memory tree.
template <int NV>
__device__ void block_partials(double (&v)[NV], double* out) {
    __shared__ double sh[NV][kHBlock];
    for (int k = 0; k < NV; k++) sh[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int w = kHBlock / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < NV; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < NV; k++) out[blockIdx.x * NV + k] = sh[k][0];
}

// y = M x for a CSR block (rows in order, entries in row order).
__global__ void __launch_bounds__(kHBlock) rows_apply(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                                                      const double* __restrict__ v, const double* __restrict__ x,
                                                      double* __restrict__ y) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        double s = 0.;
        for (int d = rp[c]; d < rp[c + 1]; d++) s += v[d] * x[ci[d]];
        y[c] = s;
    }
}

struct Blocks {
    const int *Br, *Bc, *Cr, *Cc;
    const double *Bv, *Cv;
};

// :137-149: res = b - sign B aux2 - C x, dir = res
__global__ void __launch_bounds__(kHBlock) restart_residual(int N, Blocks m, const double* __restrict__ aux2,
                                                            const double* __restrict__ x, const double* __restrict__ b,
                                                            double* __restrict__ res, double* __restrict__ dir) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
        double r = b[c];
        for (int d = m.Br[c]; d < m.Br[c + 1]; d++) r -= kSignA * m.Bv[d] * aux2[m.Bc[d]];
        for (int d = m.Cr[c]; d < m.Cr[c + 1]; d++) r -= m.Cv[d] * x[m.Cc[d]];
        res[c] = r;
        dir[c] = r;
    }
}

// :183-197: Mdir = sign B aux2 + C dir, Mres = Mdir; partials of Mdir.res and Mdir.Mdir
__global__ void __launch_bounds__(kHBlock) restart_mdir(int N, Blocks m, const double* __restrict__ aux2,
                                                        const double* __restrict__ dir, const double* __restrict__ res,
                                                        double* __restrict__ Mdir, double* __restrict__ Mres,
                                                        double* __restrict__ part) {
    double acc[2] = {0., 0.};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
        double md = 0.;
        for (int d = m.Br[c]; d < m.Br[c + 1]; d++) md += kSignA * m.Bv[d] * aux2[m.Bc[d]];
        for (int d = m.Cr[c]; d < m.Cr[c + 1]; d++) md += m.Cv[d] * dir[m.Cc[d]];
        Mdir[c] = md;
        Mres[c] = md;
        acc[0] += md * res[c];
        acc[1] += md * md;
    }
    block_partials<2>(acc, part);
}

// :280-300: vil = sign B aux2 + C Mdir; x, res, Mres updated; partials of Mres.res
__global__ void __launch_bounds__(kHBlock) iterate_update(int N, Blocks m, const double* __restrict__ aux2,
                                                          const double* __restrict__ Mdir, double alpha,
                                                          double* __restrict__ x, const double* __restrict__ dir,
                                                          double* __restrict__ res, double* __restrict__ Mres,
                                                          double* __restrict__ vil, double* __restrict__ part) {
    double acc[1] = {0.};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
        double vl = 0.;
        for (int d = m.Br[c]; d < m.Br[c + 1]; d++) vl += kSignA * m.Bv[d] * aux2[m.Bc[d]];
        for (int d = m.Cr[c]; d < m.Cr[c + 1]; d++) vl += m.Cv[d] * Mdir[m.Cc[d]];
        vil[c] = vl;
        x[c] = x[c] + alpha * dir[c];
        const double r = res[c] - alpha * Mdir[c];
        res[c] = r;
        const double mr = Mres[c] - alpha * vl;
        Mres[c] = mr;
        acc[0] += mr * r;
    }
    block_partials<1>(acc, part);
}

// :304-318: dir = res + beta dir, Mdir = Mres + beta Mdir; partials of Mdir.Mdir
__global__ void __launch_bounds__(kHBlock) iterate_directions(int N, double beta, const double* __restrict__ res,
                                                              double* __restrict__ dir, const double* __restrict__ Mres,
                                                              double* __restrict__ Mdir, double* __restrict__ part) {
    double acc[1] = {0.};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
        dir[c] = res[c] + beta * dir[c];
        const double md = Mres[c] + beta * Mdir[c];
        Mdir[c] = md;
        acc[0] += md * md;
    }
    block_partials<1>(acc, part);
}

struct HodgeRun {
    DevArena m;
    feec_system* sa = nullptr;
    ~HodgeRun() {
        m.release();
        if (sa) feec_system_destroy(sa);
    }
};

const char* hodge_title(int variant) {
    return variant == 0 ? "Hodge Conjugate Residual (diag) CSR"
         : variant == 1 ? "Hodge Conjugate Residual (SSOR) CSR" : "Hodge Conjugate Residual (textbook) CSR";
}

int hodge_cr(int variant, int N, int L, double* x, const double* b, const int* Ar, const int* Ac, const double* Av,
             const int* Br, const int* Bc, const double* Bv, const int* Btr, const int* Btc, const double* Btv,
             const int* Cr, const int* Cc, const double* Cv, double* res, double precision, int print_modulo,
             double inner_precision, feec_solve_info* info) {
    if (info) {
        *info = feec_solve_info{};
        info->true_relres = -1.0;
        info->outer_iterations = 1;
    }
    // the reference asserts these (:76-94)
    if (N <= 0 || L <= 0 || !x || !b || !res || !Ar || !Ac || !Av || !Br || !Bc || !Bv || !Btr || !Btc || !Btv ||
        !Cr || !Cc || !Cv || !(precision > 0.0) || !(inner_precision > 0.0))
        return FEEC_BADARG;
    const auto t0 = std::chrono::steady_clock::now();
    double tolerance = 0.;                                  // :97-100, serial as the reference
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = std::max(precision * std::sqrt(tolerance), kDesired);
    if (print_modulo >= -1) std::printf("(%d/%d)     BEGIN: %s\n", 0, N, hodge_title(variant));

    HodgeRun run;
    int st = feec_system_create(&run.sa, L, Ar, Ac, Av, 1, nullptr);   // validates A
    if (st != FEEC_OK) return st;
    // the diagonal as the reference sums it (:76-91), inverted for the diagonal variant
    std::vector<double> diag((size_t)L, 0.0);
    for (int c = 0; c < L; c++) {
        for (int d = Ar[c]; d < Ar[c + 1]; d++)
            if (Ac[d] == c) diag[c] += Av[d];
        if (variant == 0) diag[c] = 1. / diag[c];
    }
    int method = FEEC_METHOD_CG;
    if (variant == 0) { method = FEEC_METHOD_DIAGONAL; st = feec_system_set_diagonal_precon(run.sa, diag.data(), 1); }
    else if (variant == 1) { method = FEEC_METHOD_SSOR; st = feec_system_set_ssor(run.sa, diag.data(), 1.0, 1); }
    if (st != FEEC_OK) return st;
    cudaStream_t s = run.sa->stream;
    run.m.stream = s;

    const int nb = Br[N], nbt = Btr[L], nc = Cr[N];
    if (nb < 0 || nbt < 0 || nc < 0) return FEEC_BADARG;
    int *dBr, *dBc, *dBtr, *dBtc, *dCr, *dCc, *bad;
    double *dBv, *dBtv, *dCv, *dx, *db, *dres, *dir, *Mdir, *Mres, *vil, *aux1, *aux2, *auxR, *part, *hpart;
    FEEC_TRY(run.m.alloc(dBr, (size_t)N + 1)); FEEC_TRY(run.m.alloc(dBc, (size_t)nb)); FEEC_TRY(run.m.alloc(dBv, (size_t)nb));
    FEEC_TRY(run.m.alloc(dBtr, (size_t)L + 1)); FEEC_TRY(run.m.alloc(dBtc, (size_t)nbt)); FEEC_TRY(run.m.alloc(dBtv, (size_t)nbt));
    FEEC_TRY(run.m.alloc(dCr, (size_t)N + 1)); FEEC_TRY(run.m.alloc(dCc, (size_t)nc)); FEEC_TRY(run.m.alloc(dCv, (size_t)nc));
    FEEC_TRY(run.m.alloc(bad, 1));
    for (double** p : {&dx, &db, &dres, &dir, &Mdir, &Mres, &vil}) FEEC_TRY(run.m.alloc(*p, (size_t)N));
    for (double** p : {&aux1, &aux2, &auxR}) FEEC_TRY(run.m.alloc(*p, (size_t)L));
    const int gN = hgrid(N, 1024), gL = hgrid(L, 4096);
    FEEC_TRY(run.m.alloc(part, (size_t)2 * gN));
    std::vector<double> hp((size_t)2 * gN);
    hpart = hp.data();
    auto up = [&](auto* d, const auto* h, size_t n) {
        return n ? cudaMemcpyAsync(d, h, sizeof(*h) * n, cudaMemcpyHostToDevice, s) : cudaSuccess;
    };
    FEEC_TRY(up(dBr, Br, (size_t)N + 1)); FEEC_TRY(up(dBc, Bc, (size_t)nb)); FEEC_TRY(up(dBv, Bv, (size_t)nb));
    FEEC_TRY(up(dBtr, Btr, (size_t)L + 1)); FEEC_TRY(up(dBtc, Btc, (size_t)nbt)); FEEC_TRY(up(dBtv, Btv, (size_t)nbt));
    FEEC_TRY(up(dCr, Cr, (size_t)N + 1)); FEEC_TRY(up(dCc, Cc, (size_t)nc)); FEEC_TRY(up(dCv, Cv, (size_t)nc));
    FEEC_TRY(up(dx, x, (size_t)N)); FEEC_TRY(up(db, b, (size_t)N));
    // B, Bt and C index vectors through their columns: checked on the device first
    FEEC_TRY(cudaMemsetAsync(bad, 0, sizeof(int), s));
    FEEC_TRY(launch_validate_csr_cols(N, L, nb, dBr, dBc, bad, s));
    FEEC_TRY(launch_validate_csr_cols(L, N, nbt, dBtr, dBtc, bad, s));
    FEEC_TRY(launch_validate_csr_cols(N, N, nc, dCr, dCc, bad, s));
    int hbad = 0;
    FEEC_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));
    if (hbad) return FEEC_BADARG;

    const Blocks mb{dBr, dBc, dCr, dCc, dBv, dCv};
    int inner_total = 0;
    auto inner = [&](bool from_zero) -> int {                 // aux2 = A^-1 aux1 (approximately)
        if (from_zero) FEEC_TRY(cudaMemsetAsync(aux2, 0, sizeof(double) * (size_t)L, s));
        feec_solve_info ii;
        const int r = feec_system_solve(run.sa, method, FEEC_MODE_REFERENCE, aux2, aux1, auxR, inner_precision, 0,
                                        &ii, nullptr);
        inner_total += ii.iterations;
        // the reference ignores the inner solver's outcome; only a failed launch stops the solve
        return (r == FEEC_OK || r == FEEC_BREAKDOWN || r == FEEC_SMALL_ENERGY || r == FEEC_MAXITER) ? FEEC_OK : r;
    };
    auto sums = [&](int nv, double* out) -> int {              // fixed-order host sum of block partials
        FEEC_TRY(cudaMemcpyAsync(hpart, part, sizeof(double) * (size_t)nv * gN, cudaMemcpyDeviceToHost, s));
        FEEC_TRY(cudaStreamSynchronize(s));
        for (int k = 0; k < nv; k++) {
            double a = 0.;
            for (int i = 0; i < gN; i++) a += hpart[(size_t)i * nv + k];
            out[k] = a;
        }
        return FEEC_OK;
    };
    auto launched = [&]() { note_launch(); return cudaGetLastError(); };

    // restart (:107-200)
    rows_apply<<<gL, kHBlock, 0, s>>>(L, dBtr, dBtc, dBtv, dx, aux1);
    FEEC_TRY(launched());
    if ((st = inner(true)) != FEEC_OK) return st;
    restart_residual<<<gN, kHBlock, 0, s>>>(N, mb, aux2, dx, db, dres, dir);
    FEEC_TRY(launched());
    rows_apply<<<gL, kHBlock, 0, s>>>(L, dBtr, dBtc, dBtv, dir, aux1);
    FEEC_TRY(launched());
    if ((st = inner(true)) != FEEC_OK) return st;
    restart_mdir<<<gN, kHBlock, 0, s>>>(N, mb, aux2, dir, dres, Mdir, Mres, part);
    FEEC_TRY(launched());
    double v2[2];
    if ((st = sums(2, v2)) != FEEC_OK) return st;
    double Md_r = v2[0], Md_Md = v2[1];

    int K = 0, status = FEEC_MAXITER;
    while (K < N) {
        if (print_modulo > 0 && K % print_modulo == 0)
            std::printf("(%d/%d)   INTERIM: Residual norm is %.9le < %.9le\n", K, N, std::sqrt(Md_r), tolerance);
        if (!std::isfinite(Md_r) || Md_r < 0.) {               // :212-218
            if (print_modulo >= -2 || variant == 1)
                std::printf("(%d/%d) BREAKDOWN: Residual energy is unreasonable with %.9le\n", K, N, Md_r);
            status = FEEC_BREAKDOWN; break;
        }
        if (std::fabs(Md_r) < tolerance * tolerance) { status = FEEC_OK; break; }
        if (!std::isfinite(Md_Md) || Md_Md < 0.) {             // :224-232
            if (print_modulo >= -2 || variant == 1)
                std::printf("(%d/%d) BREAKDOWN: Gradient double energy is unreasonable with %.9le\n", K, N, Md_Md);
            status = FEEC_BREAKDOWN; break;
        }
        if (std::sqrt(std::fabs(Md_Md)) < kEpsilon) {          // :233-238
            if (print_modulo >= -2 || variant == 1)
                std::printf("(%d/%d)   WARNING: Gradient double energy is small with %.9le\n", K, N, Md_Md);
            status = FEEC_SMALL_ENERGY; break;
        }
        const double alpha = Md_r / Md_Md;                      // :242
        rows_apply<<<gL, kHBlock, 0, s>>>(L, dBtr, dBtc, dBtv, Mdir, aux1);
        FEEC_TRY(launched());
        if ((st = inner(false)) != FEEC_OK) return st;
        iterate_update<<<gN, kHBlock, 0, s>>>(N, mb, aux2, Mdir, alpha, dx, dir, dres, Mres, vil, part);
        FEEC_TRY(launched());
        double v1[1];
        if ((st = sums(1, v1)) != FEEC_OK) return st;
        const double new_Mr_r = v1[0];
        const double beta = new_Mr_r / Md_r;                    // :302
        iterate_directions<<<gN, kHBlock, 0, s>>>(N, beta, dres, dir, Mres, Mdir, part);
        FEEC_TRY(launched());
        if ((st = sums(1, v1)) != FEEC_OK) return st;
        Md_Md = v1[0];
        Md_r = new_Mr_r;
        K++;
    }
    FEEC_TRY(cudaMemcpyAsync(x, dx, sizeof(double) * (size_t)N, cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaMemcpyAsync(res, dres, sizeof(double) * (size_t)N, cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));
    const bool finish = variant == 1 ? print_modulo >= 0 : print_modulo >= -1;   // :321 / :324
    if (finish)
        std::printf("(%d/%d) %9s: Residual norm is %.9le < %.9le\n", K, N,
                    std::sqrt(Md_r) < tolerance ? "SUCCESS" : "FAILED", std::sqrt(Md_r), tolerance);
    if (info) {
        info->status = status;
        info->iterations = K;
        info->outer_iterations = inner_total;
        info->tolerance = tolerance;
        info->final_norm = std::sqrt(std::fabs(Md_r));
        info->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return status;
}

}  // namespace
}  // namespace feec

using namespace feec;

extern "C" {

#define FEEC_HODGE_ARGS                                                                                         \
    int N, int L, double* x, const double* b, const int* Arows, const int* Acolumns, const double* Avalues,       \
        const int* Brows, const int* Bcolumns, const double* Bvalues, const int* Btrows, const int* Btcolumns,    \
        const double* Btvalues, const int* Crows, const int* Ccolumns, const double* Cvalues, double* residual,    \
        double precision, int print_modulo, double inner_precision, int inner_print_modulo, feec_solve_info* info
#define FEEC_HODGE_PASS                                                                                         \
    N, L, x, b, Arows, Acolumns, Avalues, Brows, Bcolumns, Bvalues, Btrows, Btcolumns, Btvalues, Crows, Ccolumns, \
        Cvalues, residual, precision, print_modulo, inner_precision, info

int feec_hodge_cr_csr(FEEC_HODGE_ARGS) {
    (void)inner_print_modulo;
    return hodge_cr(1, FEEC_HODGE_PASS);
}

int feec_hodge_cr_csr_diagonal(FEEC_HODGE_ARGS) {
    (void)inner_print_modulo;
    return hodge_cr(0, FEEC_HODGE_PASS);
}

int feec_hodge_cr_csr_ssor(FEEC_HODGE_ARGS) {
    (void)inner_print_modulo;
    return hodge_cr(1, FEEC_HODGE_PASS);
}

int feec_hodge_cr_csr_textbook(FEEC_HODGE_ARGS) {
    (void)inner_print_modulo;
    return hodge_cr(2, FEEC_HODGE_PASS);
}

}  // extern "C"
