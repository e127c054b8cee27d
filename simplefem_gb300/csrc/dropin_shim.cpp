// libfeec_dropin.so: exports the reference's own C++ entry points of the CSR
// Krylov path (solver/sparsesolver.hpp:11-19, 21-31, 33-43, 46-56, 59-70, 73-84, 89-139, and
// solver/systemsparsesolver.hpp:10-72, with Float =
// double, the reference's default build) so that an application linked
// against FEEC++'s solver module can link this library instead and run the
// solves on the GPU unchanged. Each function forwards to the C ABI and returns
// the iteration count K exactly as the reference does.
//
// Error behaviour: the reference guards its arguments with assert()
// (sparsesolver.cpp:32-43), which aborts in checked builds. A rejected argument
// or a CUDA failure here prints a message and aborts likewise; numerical
// breakdowns return the current K after the reference's log lines.
#include <cstdio>
#include <cstdlib>

#include "feec_gpu.h"

namespace {

int checked(int status, const feec_solve_info& info, const char* fn) {
    switch (status) {
        case FEEC_OK:
        case FEEC_BREAKDOWN:
        case FEEC_SMALL_ENERGY:
        case FEEC_MAXITER:
            return info.iterations;
        default:
            std::fprintf(stderr, "%s: %s (status %d)\n", fn, feec_status_string(status), status);
            std::abort();
    }
}

}  // namespace

int ConjugateGradientSolverCSR(const int N, double* x, const double* b, const int* csrrows, const int* csrcolumns,
                               const double* csrvalues, double* residual, double precision, int print_modulo) {
    feec_solve_info info;
    const int st = feec_cg_csr(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision, print_modulo, &info);
    return checked(st, info, "ConjugateGradientSolverCSR");
}

int ConjugateGradientSolverCSR_SSOR(const int N, double* x, const double* b, const int* csrrows,
                                    const int* csrcolumns, const double* csrvalues, double* residual,
                                    double precision, int print_modulo, const double* diagonal, double omega) {
    feec_solve_info info;
    const int st = feec_cg_csr_ssor(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision, print_modulo,
                                    diagonal, omega, &info);
    return checked(st, info, "ConjugateGradientSolverCSR_SSOR");
}

int ConjugateGradientSolverCSR_Rainbow(const int N, double* x, const double* b, const int* csrrows,
                                       const int* csrcolumns, const double* csrvalues, double* residual,
                                       double precision, int print_modulo, const double* diagonal, double omega,
                                       int num_colors, const int* F, const int* B, const int* R) {
    feec_solve_info info;
    const int st = feec_cg_csr_rainbow(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision, print_modulo,
                                       diagonal, omega, num_colors, F, B, R, &info);
    return checked(st, info, "ConjugateGradientSolverCSR_Rainbow");
}

int ConjugateGradientSolverCSR_SSOR_Eisenstat(const int N, double* x, const double* b, const int* csrrows,
                                              const int* csrcolumns, const double* csrvalues, double* residual,
                                              double precision, int print_modulo, const double* diagonal,
                                              double omega) {
    feec_solve_info info;
    const int st = feec_cg_csr_ssor_eisenstat(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision,
                                              print_modulo, diagonal, omega, &info);
    return checked(st, info, "ConjugateGradientSolverCSR_SSOR_Eisenstat");
}

int ConjugateGradientSolverCSR_Eisenstat_Rainbow(const int N, double* x, const double* b, const int* csrrows,
                                                 const int* csrcolumns, const double* csrvalues, double* residual,
                                                 double precision, int print_modulo, const double* diagonal,
                                                 double omega, int num_colors, const int* F, const int* B,
                                                 const int* R) {
    feec_solve_info info;
    const int st = feec_cg_csr_eisenstat_rainbow(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision,
                                                 print_modulo, diagonal, omega, num_colors, F, B, R, &info);
    return checked(st, info, "ConjugateGradientSolverCSR_Eisenstat_Rainbow");
}

int ConjugateGradientSolverCSR_DiagonalPreconditioner(const int N, double* x, const double* b, const int* csrrows,
                                                      const int* csrcolumns, const double* csrvalues,
                                                      double* residual, double precision, int print_modulo,
                                                      const double* precon) {
    feec_solve_info info;
    const int st = feec_cg_csr_diagonal_precon(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision,
                                               print_modulo, precon, &info);
    return checked(st, info, "ConjugateGradientSolverCSR_DiagonalPreconditioner");
}

// solver/sparsesolver.hpp:89-139: conjugate residuals, MINRES and the diagonally
// preconditioned Chebyshev iteration.
int ConjugateResidualSolverCSR(const int N, double* x, const double* b, const int* csrrows, const int* csrcolumns,
                               const double* csrvalues, double* residual, double precision, int print_modulo) {
    feec_solve_info info;
    const int st = feec_cr_csr(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision, print_modulo, &info);
    return checked(st, info, "ConjugateResidualSolverCSR");
}

int ConjugateResidualSolverCSR_textbook(const int N, double* x, const double* b, const int* csrrows,
                                        const int* csrcolumns, const double* csrvalues, double* residual,
                                        double precision, int print_modulo) {
    feec_solve_info info;
    const int st = feec_cr_csr_textbook(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision, print_modulo,
                                        &info);
    return checked(st, info, "ConjugateResidualSolverCSR_textbook");
}

int MINRESCSR(const int N, double* x, const double* b, const int* csrrows, const int* csrcolumns,
              const double* csrvalues, double* res, const double precision, int print_modulo) {
    feec_solve_info info;
    const int st = feec_minres_csr(N, x, b, csrrows, csrcolumns, csrvalues, res, precision, print_modulo, &info);
    return checked(st, info, "MINRESCSR");
}

int ChebyshevIteration_DiagonalPreconditioner(const int N, double* x, const double* b, const int* csrrows,
                                              const int* csrcolumns, const double* csrvalues, double* residual,
                                              const double precision, int print_modulo, const double* precon,
                                              const double lower, const double upper) {
    feec_solve_info info;
    const int st = feec_chebyshev_diag(N, x, b, csrrows, csrcolumns, csrvalues, residual, precision, print_modulo,
                                       precon, lower, upper, &info);
    return checked(st, info, "ChebyshevIteration_DiagonalPreconditioner");
}

// solver/systemsparsesolver.hpp:10-72: the Hodge conjugate residual solvers.
#define FEEC_SHIM_HODGE(name, entry)                                                                          \
    int name(const int N, const int L, double* x, const double* b, const int* Arows, const int* Acolumns,       \
             const double* Avalues, const int* Brows, const int* Bcolumns, const double* Bvalues,               \
             const int* Btrows, const int* Btcolumns, const double* Btvalues, const int* Crows,                 \
             const int* Ccolumns, const double* Cvalues, double* residual, double precision, int print_modulo,  \
             double inneriteration_precision, int inneriteration_print_modulo) {                                \
        feec_solve_info info;                                                                                   \
        const int st = entry(N, L, x, b, Arows, Acolumns, Avalues, Brows, Bcolumns, Bvalues, Btrows, Btcolumns, \
                             Btvalues, Crows, Ccolumns, Cvalues, residual, precision, print_modulo,              \
                             inneriteration_precision, inneriteration_print_modulo, &info);                     \
        return checked(st, info, #name);                                                                        \
    }
FEEC_SHIM_HODGE(HodgeConjugateResidualSolverCSR, feec_hodge_cr_csr)
FEEC_SHIM_HODGE(HodgeConjugateResidualSolverCSR_diagonal, feec_hodge_cr_csr_diagonal)
FEEC_SHIM_HODGE(HodgeConjugateResidualSolverCSR_SSOR, feec_hodge_cr_csr_ssor)
FEEC_SHIM_HODGE(HodgeConjugateResidualSolverCSR_textbook, feec_hodge_cr_csr_textbook)

int HodgeHerzogSoodhalterMethod(const int dimension_A, const int dimension_C, double* x_A, double* x_C,
                                const double* b_A, const double* b_C, const int* Arows, const int* Acolumns,
                                const double* Avalues, const int* Brows, const int* Bcolumns, const double* Bvalues,
                                const int* Btrows, const int* Btcolumns, const double* Btvalues, const int* Crows,
                                const int* Ccolumns, const double* Cvalues, double precision, int print_modulo,
                                const int* PArows, const int* PAcolumns, const double* PAvalues, const int* PCrows,
                                const int* PCcolumns, const double* PCvalues, double inneriteration_precision,
                                int inneriteration_print_modulo) {
    feec_solve_info info;
    const int st = feec_hodge_herzog_soodhalter(dimension_A, dimension_C, x_A, x_C, b_A, b_C, Arows, Acolumns, Avalues,
                                                Brows, Bcolumns, Bvalues, Btrows, Btcolumns, Btvalues, Crows, Ccolumns,
                                                Cvalues, precision, print_modulo, PArows, PAcolumns, PAvalues, PCrows,
                                                PCcolumns, PCvalues, inneriteration_precision,
                                                inneriteration_print_modulo, &info);
    return checked(st, info, "HodgeHerzogSoodhalterMethod");
}
