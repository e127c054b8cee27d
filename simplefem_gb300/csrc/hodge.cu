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
// and HodgeHerzogSoodhalterMethod (:1122-1575): preconditioned MINRES on the saddle-point
// system [[-A, Bt], [B, C]] with the block preconditioner diag(PA, PC) applied by inner CG
// solves (each block optional).
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

// ---- Herzog-Soodhalter block MINRES: row kernels of the A part (rows of A and Bt) and
// the C part (rows of B and C) --------------------------------------------------------

struct Pair {            // two CSR blocks applied to (xa, xc) row by row
    const int *r1, *c1, *r2, *c2;
    const double *v1, *v2;
};

// :1246-1257: v1 = b + s1 M1 xa + s2 M2 xc (s1, s2 = +-1 as the block's signs); v0 = w0 = w1 = 0; z = v1
__global__ void __launch_bounds__(kHBlock) hhs_restart(int n, Pair m, double s1, double s2, const double* __restrict__ xa,
                                                       const double* __restrict__ xc, const double* __restrict__ b,
                                                       double* __restrict__ v0, double* __restrict__ w0,
                                                       double* __restrict__ w1, double* __restrict__ v1,
                                                       double* __restrict__ z) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        v0[r] = 0.; w0[r] = 0.; w1[r] = 0.;
        double v = b[r];
        for (int d = m.r1[r]; d < m.r1[r + 1]; d++) v += s1 * m.v1[d] * xa[m.c1[d]];
        for (int d = m.r2[r]; d < m.r2[r + 1]; d++) v += s2 * m.v2[d] * xc[m.c2[d]];
        v1[r] = v;
        z[r] = v;
    }
}

__global__ void __launch_bounds__(kHBlock) dot_partials(int n, const double* __restrict__ a,
                                                        const double* __restrict__ b, double* __restrict__ part) {
    double acc[1] = {0.};
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) acc[0] += a[r] * b[r];
    block_partials<1>(acc, part);
}

// :1314-1322: v1 /= gamma, z /= gamma, m = v1
__global__ void __launch_bounds__(kHBlock) hhs_scale(int n, double gamma, double* __restrict__ v1,
                                                     double* __restrict__ z, double* __restrict__ mm) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const double v = v1[r] / gamma;
        v1[r] = v;
        z[r] = z[r] / gamma;
        mm[r] = v;
    }
}

// :1345-1371: p = s1 M1 za + s2 M2 zc (accumulated from 0 in that order); partials of p.z_own
__global__ void __launch_bounds__(kHBlock) hhs_product(int n, Pair m, double s1, double s2,
                                                       const double* __restrict__ za, const double* __restrict__ zc,
                                                       const double* __restrict__ zown, double* __restrict__ p,
                                                       double* __restrict__ part) {
    double acc[1] = {0.};
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        double v = 0.;
        for (int d = m.r1[r]; d < m.r1[r + 1]; d++) v += s1 * m.v1[d] * za[m.c1[d]];
        for (int d = m.r2[r]; d < m.r2[r + 1]; d++) v += s2 * m.v2[d] * zc[m.c2[d]];
        p[r] = v;
        acc[0] += v * zown[r];
    }
    block_partials<1>(acc, part);
}

// :1373-1387: vn = p - delta v1 - gamma v0, zn = vn; partials of zn.vn
__global__ void __launch_bounds__(kHBlock) hhs_lanczos(int n, double delta, double gamma, const double* __restrict__ p,
                                                       const double* __restrict__ v1, const double* __restrict__ v0,
                                                       double* __restrict__ vn, double* __restrict__ zn,
                                                       double* __restrict__ part) {
    double acc[1] = {0.};
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const double v = p[r] - delta * v1[r] - gamma * v0[r];
        vn[r] = v;
        zn[r] = v;
        acc[0] += v * v;
    }
    block_partials<1>(acc, part);
}

struct HhsStep {
    double gamma_n, sn, cn, a1, a2, a3, ce;   // ce = cn * eta
};

// :1447-1474: vn, zn scaled by 1/gamma_n; partials of m.zn (theta) and zn.vn (psi) with the
// old m; then m = -sn m + cn vn, wn = (z - a3 w0 - a2 w1) / a1, x = x + cn eta wn
__global__ void __launch_bounds__(kHBlock) hhs_rotate(int n, HhsStep q, double* __restrict__ vn, double* __restrict__ zn,
                                                      double* __restrict__ mm, const double* __restrict__ z,
                                                      const double* __restrict__ w0, const double* __restrict__ w1,
                                                      double* __restrict__ wn, double* __restrict__ x,
                                                      double* __restrict__ part) {
    double acc[2] = {0., 0.};
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const double v = vn[r] / q.gamma_n;
        const double zz = zn[r] / q.gamma_n;
        vn[r] = v;
        zn[r] = zz;
        acc[0] += mm[r] * zz;
        acc[1] += zz * v;
        mm[r] = -q.sn * mm[r] + q.cn * v;
        const double w = (z[r] - q.a3 * w0[r] - q.a2 * w1[r]) / q.a1;
        wn[r] = w;
        x[r] = x[r] + q.ce * w;
    }
    block_partials<2>(acc, part);
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
        info->error_estimate = -1.0;
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

struct HhsRun {
    DevArena m;
    feec_system* pa = nullptr;
    feec_system* pc = nullptr;
    ~HhsRun() {
        m.release();
        if (pa) feec_system_destroy(pa);
        if (pc) feec_system_destroy(pc);
    }
};

int hodge_hs(int dA, int dC, double* x_A, double* x_C, const double* b_A, const double* b_C, const int* Ar,
             const int* Ac, const double* Av, const int* Br, const int* Bc, const double* Bv, const int* Btr,
             const int* Btc, const double* Btv, const int* Cr, const int* Cc, const double* Cv, double precision,
             int print_modulo, const int* PAr, const int* PAc, const double* PAv, const int* PCr, const int* PCc,
             const double* PCv, double inner_precision, feec_solve_info* info) {
    if (info) {
        *info = feec_solve_info{};
        info->true_relres = -1.0;
        info->error_estimate = -1.0;
        info->outer_iterations = 1;
    }
    // the reference asserts these (:1142-1159)
    if (dA <= 0 || dC <= 0 || !x_A || !x_C || !b_A || !b_C || !Ar || !Ac || !Av || !Br || !Bc || !Bv || !Btr ||
        !Btc || !Btv || !Cr || !Cc || !Cv || !(precision > 0.0) || !(inner_precision > 0.0))
        return FEEC_BADARG;
    const auto t0 = std::chrono::steady_clock::now();
    double tolerance = 0.;                                 // :1167-1171
    for (int i = 0; i < dA; i++) tolerance += b_A[i] * b_A[i];
    for (int i = 0; i < dC; i++) tolerance += b_C[i] * b_C[i];
    tolerance = std::max(precision * std::sqrt(tolerance), kDesired);
    const int max_count = dA + dC;
    const bool use_pa = PAr && PAc && PAv, use_pc = PCr && PCc && PCv;
    if (print_modulo >= -1) {
        std::printf("(%d/%d)     BEGIN: Hodge Herzog-Soodhalter CSR\n", 0, max_count);
        if (use_pa) std::printf("      Preconditioner for A detected\n");
        if (use_pc) std::printf("      Preconditioner for C detected\n");
    }
    HhsRun run;
    int st;
    if (use_pa && (st = feec_system_create(&run.pa, dA, PAr, PAc, PAv, 1, nullptr)) != FEEC_OK) return st;
    if (use_pc && (st = feec_system_create(&run.pc, dC, PCr, PCc, PCv, 1, nullptr)) != FEEC_OK) return st;
    cudaStream_t s = nullptr;                                // CUDA's default stream, as the systems'
    run.m.stream = s;
    const int na = Ar[dA], nbt = Btr[dA], nb = Br[dC], nc = Cr[dC];
    if (na < 0 || nbt < 0 || nb < 0 || nc < 0) return FEEC_BADARG;
    int *dAr, *dAc, *dBr, *dBc, *dBtr, *dBtc, *dCr, *dCc, *bad;
    double *dAv, *dBv, *dBtv, *dCv, *part;
    FEEC_TRY(run.m.alloc(dAr, (size_t)dA + 1)); FEEC_TRY(run.m.alloc(dAc, (size_t)na)); FEEC_TRY(run.m.alloc(dAv, (size_t)na));
    FEEC_TRY(run.m.alloc(dBtr, (size_t)dA + 1)); FEEC_TRY(run.m.alloc(dBtc, (size_t)nbt)); FEEC_TRY(run.m.alloc(dBtv, (size_t)nbt));
    FEEC_TRY(run.m.alloc(dBr, (size_t)dC + 1)); FEEC_TRY(run.m.alloc(dBc, (size_t)nb)); FEEC_TRY(run.m.alloc(dBv, (size_t)nb));
    FEEC_TRY(run.m.alloc(dCr, (size_t)dC + 1)); FEEC_TRY(run.m.alloc(dCc, (size_t)nc)); FEEC_TRY(run.m.alloc(dCv, (size_t)nc));
    FEEC_TRY(run.m.alloc(bad, 1));
    // A part: x, b, v0, v1, vn, w0, w1, wn, z, zn, m, p (indices 0..11); C part likewise
    double* va[12];
    double* vc[12];
    for (int k = 0; k < 12; k++) { FEEC_TRY(run.m.alloc(va[k], (size_t)dA)); FEEC_TRY(run.m.alloc(vc[k], (size_t)dC)); }
    const int gA = hgrid(dA, 1024), gC = hgrid(dC, 1024), gmax = std::max(gA, gC);
    FEEC_TRY(run.m.alloc(part, (size_t)2 * gmax));
    std::vector<double> hp((size_t)2 * gmax);
    auto up = [&](auto* d, const auto* h, size_t n) {
        return n ? cudaMemcpyAsync(d, h, sizeof(*h) * n, cudaMemcpyHostToDevice, s) : cudaSuccess;
    };
    FEEC_TRY(up(dAr, Ar, (size_t)dA + 1)); FEEC_TRY(up(dAc, Ac, (size_t)na)); FEEC_TRY(up(dAv, Av, (size_t)na));
    FEEC_TRY(up(dBtr, Btr, (size_t)dA + 1)); FEEC_TRY(up(dBtc, Btc, (size_t)nbt)); FEEC_TRY(up(dBtv, Btv, (size_t)nbt));
    FEEC_TRY(up(dBr, Br, (size_t)dC + 1)); FEEC_TRY(up(dBc, Bc, (size_t)nb)); FEEC_TRY(up(dBv, Bv, (size_t)nb));
    FEEC_TRY(up(dCr, Cr, (size_t)dC + 1)); FEEC_TRY(up(dCc, Cc, (size_t)nc)); FEEC_TRY(up(dCv, Cv, (size_t)nc));
    FEEC_TRY(up(va[0], x_A, (size_t)dA)); FEEC_TRY(up(va[1], b_A, (size_t)dA));
    FEEC_TRY(up(vc[0], x_C, (size_t)dC)); FEEC_TRY(up(vc[1], b_C, (size_t)dC));
    FEEC_TRY(cudaMemsetAsync(bad, 0, sizeof(int), s));
    FEEC_TRY(launch_validate_csr_cols(dA, dA, na, dAr, dAc, bad, s));
    FEEC_TRY(launch_validate_csr_cols(dA, dC, nbt, dBtr, dBtc, bad, s));
    FEEC_TRY(launch_validate_csr_cols(dC, dA, nb, dBr, dBc, bad, s));
    FEEC_TRY(launch_validate_csr_cols(dC, dC, nc, dCr, dCc, bad, s));
    int hbad = 0;
    FEEC_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));
    if (hbad) return FEEC_BADARG;

    double *xA = va[0], *bA = va[1], *v0A = va[2], *v1A = va[3], *vnA = va[4], *w0A = va[5], *w1A = va[6];
    double *wnA = va[7], *zA = va[8], *znA = va[9], *mA = va[10], *pA = va[11];
    double *xC = vc[0], *bC = vc[1], *v0C = vc[2], *v1C = vc[3], *vnC = vc[4], *w0C = vc[5], *w1C = vc[6];
    double *wnC = vc[7], *zC = vc[8], *znC = vc[9], *mC = vc[10], *pC = vc[11];
    const Pair rowsA{dAr, dAc, dBtr, dBtc, dAv, dBtv};      // A part: rows of A and of Bt
    const Pair rowsC{dBr, dBc, dCr, dCc, dBv, dCv};         // C part: rows of B and of C
    int inner_total = 0;
    auto precon = [&](feec_system* P, double* z, const double* v, double* r) -> int {
        feec_solve_info ii;
        const int e = feec_system_solve(P, FEEC_METHOD_CG, FEEC_MODE_REFERENCE, z, v, r, inner_precision, 0, &ii,
                                        nullptr);
        inner_total += ii.iterations;
        return (e == FEEC_OK || e == FEEC_BREAKDOWN || e == FEEC_SMALL_ENERGY || e == FEEC_MAXITER) ? FEEC_OK : e;
    };
    auto sums = [&](int nblocks, int nv, double* out) -> int {
        FEEC_TRY(cudaMemcpyAsync(hp.data(), part, sizeof(double) * (size_t)nv * nblocks, cudaMemcpyDeviceToHost, s));
        FEEC_TRY(cudaStreamSynchronize(s));
        for (int k = 0; k < nv; k++) {
            double a = 0.;
            for (int i = 0; i < nblocks; i++) a += hp[(size_t)i * nv + k];
            out[k] = a;
        }
        return FEEC_OK;
    };
    auto dot = [&](int n, int g, const double* a, const double* b, double& out) -> int {
        dot_partials<<<g, kHBlock, 0, s>>>(n, a, b, part);
        note_launch();
        FEEC_TRY(cudaGetLastError());
        return sums(g, 1, &out);
    };

    // restart (:1240-1330)
    hhs_restart<<<gA, kHBlock, 0, s>>>(dA, rowsA, kSignA, -1., xA, xC, bA, v0A, w0A, w1A, v1A, zA);
    hhs_restart<<<gC, kHBlock, 0, s>>>(dC, rowsC, -1., -1., xA, xC, bC, v0C, w0C, w1C, v1C, zC);
    note_launch(); note_launch();
    FEEC_TRY(cudaGetLastError());
    if (use_pa && (st = precon(run.pa, zA, v1A, wnA)) != FEEC_OK) return st;
    if (use_pc && (st = precon(run.pc, zC, v1C, wnC)) != FEEC_OK) return st;
    double v1zA = 0., v1zC = 0.;
    if ((st = dot(dA, gA, v1A, zA, v1zA)) != FEEC_OK || (st = dot(dC, gC, v1C, zC, v1zC)) != FEEC_OK) return st;
    double gamma = std::sqrt(v1zA + v1zC);
    hhs_scale<<<gA, kHBlock, 0, s>>>(dA, gamma, v1A, zA, mA);
    hhs_scale<<<gC, kHBlock, 0, s>>>(dC, gamma, v1C, zC, mC);
    note_launch(); note_launch();
    FEEC_TRY(cudaGetLastError());
    const double psiA0 = v1zA / (gamma * gamma), psiC0 = v1zC / (gamma * gamma);
    double mu_A = psiA0, mu_C = psiC0, eta = gamma;
    double s0 = 0., s1 = 0., c0 = 1., c1 = 1.;
    (void)mu_A; (void)mu_C;

    int count = 0;
    while (count < max_count) {
        if (std::fabs(eta) < tolerance) break;                // :1336-1339
        double zpA = 0., zpC = 0.;
        hhs_product<<<gA, kHBlock, 0, s>>>(dA, rowsA, -kSignA, 1., zA, zC, zA, pA, part);
        note_launch();
        FEEC_TRY(cudaGetLastError());
        if ((st = sums(gA, 1, &zpA)) != FEEC_OK) return st;
        hhs_product<<<gC, kHBlock, 0, s>>>(dC, rowsC, 1., 1., zA, zC, zC, pC, part);
        note_launch();
        FEEC_TRY(cudaGetLastError());
        if ((st = sums(gC, 1, &zpC)) != FEEC_OK) return st;
        const double delta = zpA + zpC;
        double znvnA = 0., znvnC = 0.;
        hhs_lanczos<<<gA, kHBlock, 0, s>>>(dA, delta, gamma, pA, v1A, v0A, vnA, znA, part);
        note_launch();
        FEEC_TRY(cudaGetLastError());
        if ((st = sums(gA, 1, &znvnA)) != FEEC_OK) return st;
        hhs_lanczos<<<gC, kHBlock, 0, s>>>(dC, delta, gamma, pC, v1C, v0C, vnC, znC, part);
        note_launch();
        FEEC_TRY(cudaGetLastError());
        if ((st = sums(gC, 1, &znvnC)) != FEEC_OK) return st;
        if (use_pa) {
            if ((st = precon(run.pa, znA, vnA, wnA)) != FEEC_OK) return st;
            if ((st = dot(dA, gA, znA, vnA, znvnA)) != FEEC_OK) return st;
        }
        if (use_pc) {
            if ((st = precon(run.pc, znC, vnC, wnC)) != FEEC_OK) return st;
            if ((st = dot(dC, gC, znC, vnC, znvnC)) != FEEC_OK) return st;
        }
        const double gamma_n = std::sqrt(znvnA + znvnC);      // :1445
        const double alpha_0 = c1 * delta - c0 * s1 * gamma;
        const double alpha_1 = std::sqrt(alpha_0 * alpha_0 + gamma_n * gamma_n);
        const double alpha_2 = s1 * delta + c0 * c1 * gamma;
        const double alpha_3 = s0 * gamma;
        const double cn = alpha_0 / alpha_1;
        const double sn = gamma_n / alpha_1;
        const HhsStep q{gamma_n, sn, cn, alpha_1, alpha_2, alpha_3, cn * eta};
        double tpA[2], tpC[2];
        hhs_rotate<<<gA, kHBlock, 0, s>>>(dA, q, vnA, znA, mA, zA, w0A, w1A, wnA, xA, part);
        note_launch();
        FEEC_TRY(cudaGetLastError());
        if ((st = sums(gA, 2, tpA)) != FEEC_OK) return st;
        hhs_rotate<<<gC, kHBlock, 0, s>>>(dC, q, vnC, znC, mC, zC, w0C, w1C, wnC, xC, part);
        note_launch();
        FEEC_TRY(cudaGetLastError());
        if ((st = sums(gC, 2, tpC)) != FEEC_OK) return st;
        mu_A = sn * sn * mu_A - 2 * sn * cn * tpA[0] + cn * cn * tpA[1];
        mu_C = sn * sn * mu_C - 2 * sn * cn * tpC[0] + cn * cn * tpC[1];
        eta = -sn * eta;
        // :1494-1503: v0 <- v1 <- vn <- v0, w0 <- w1 <- wn <- w0, z <-> zn
        double* t;
        t = v0A; v0A = v1A; v1A = vnA; vnA = t;
        t = v0C; v0C = v1C; v1C = vnC; vnC = t;
        t = w0A; w0A = w1A; w1A = wnA; wnA = t;
        t = w0C; w0C = w1C; w1C = wnC; wnC = t;
        t = zA; zA = znA; znA = t;
        t = zC; zC = znC; znC = t;
        gamma = gamma_n;
        c0 = c1; c1 = cn;
        s0 = s1; s1 = sn;
        if (print_modulo > 0 && count % print_modulo == 0)
            std::printf("(%d/%d)   INTERIM: Residual norm is %.9le < %.9le\n", count, max_count, std::fabs(eta), tolerance);
        count++;
    }
    FEEC_TRY(cudaMemcpyAsync(x_A, xA, sizeof(double) * (size_t)dA, cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaMemcpyAsync(x_C, xC, sizeof(double) * (size_t)dC, cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));
    const double dev = std::fabs(eta);
    if (print_modulo >= -1)
        std::printf("(%d/%d) %9s: Residual norm is %.9le < %.9le\n", count, max_count,
                    dev < tolerance ? "SUCCESS" : "FAILED", dev, tolerance);
    const int status = dev < tolerance ? FEEC_OK : FEEC_MAXITER;
    if (info) {
        info->status = status;
        info->iterations = count;
        info->outer_iterations = inner_total;
        info->tolerance = tolerance;
        info->final_norm = dev;
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

int feec_hodge_herzog_soodhalter(int dimension_A, int dimension_C, double* x_A, double* x_C, const double* b_A,
                                 const double* b_C, const int* Arows, const int* Acolumns, const double* Avalues,
                                 const int* Brows, const int* Bcolumns, const double* Bvalues, const int* Btrows,
                                 const int* Btcolumns, const double* Btvalues, const int* Crows, const int* Ccolumns,
                                 const double* Cvalues, double precision, int print_modulo, const int* PArows,
                                 const int* PAcolumns, const double* PAvalues, const int* PCrows,
                                 const int* PCcolumns, const double* PCvalues, double inner_precision,
                                 int inner_print_modulo, feec_solve_info* info) {
    (void)inner_print_modulo;
    return hodge_hs(dimension_A, dimension_C, x_A, x_C, b_A, b_C, Arows, Acolumns, Avalues, Brows, Bcolumns, Bvalues,
                    Btrows, Btcolumns, Btvalues, Crows, Ccolumns, Cvalues, precision, print_modulo, PArows, PAcolumns,
                    PAvalues, PCrows, PCcolumns, PCvalues, inner_precision, info);
}

}  // extern "C"
