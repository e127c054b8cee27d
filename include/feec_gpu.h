/*
 * feec_gpu.h — C ABI of the GB300 sparse-CSR Krylov library (libfeec_gpu.so).
 *
 * Drop-in replacement for the CSR hot path of FEEC++ (martinlicht/simplefem):
 * CSR SpMV, the CG drivers of solver/sparsesolver.hpp and the Rainbow greedy
 * coloring of sparse/rainbow.hpp. Plain C types only: int32 CSR arrays
 * (A = row pointers, C = column indices, V = values, as MatrixCSR stores them,
 * sparse/matcsr.hpp:117-119) and double vectors.
 *
 * Every entry point returns a feec_status. The "host" entry points take host
 * pointers (the reference's raw-pointer convention) and copy to and from the
 * GPU inside the call; the feec_system_* entry points keep a matrix resident
 * on the GPU and take device pointers.
 *
 * Threads: the host entry points are reentrant like the reference's functions
 * (each call owns its device scratch; calls from several host threads are
 * ordered on CUDA's default stream). A feec_system or feec_batch handle is used
 * by one host thread at a time. A feec_server may be used from any number of
 * threads (its queue is locked inside). The one exception is
 * feec_cg_csr_noalloc: all its calls share one fixed device scratch array, so
 * the caller must serialise calls whose GPU work could overlap.
 */
#ifndef FEEC_GPU_H
#define FEEC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum feec_status {
    FEEC_OK = 0,             /* converged (reference stopping rule or requested rule)        */
    FEEC_BREAKDOWN = 1,      /* non-finite or negative r.r / z.r / d.Ad (sparsesolver.cpp:148-151) */
    FEEC_SMALL_ENERGY = 2,   /* sqrt|d.Ad| < machine epsilon (sparsesolver.cpp:153-157)       */
    FEEC_MAXITER = 3,        /* iteration cap reached without meeting the tolerance            */
    FEEC_TIMEOUT = 4,        /* a device-side wait gave up; the GPU context stays usable       */
    FEEC_OOM = 5,            /* device allocation failed or the memory budget was exceeded     */
    FEEC_BADARG = 6,         /* invalid argument (the reference asserts these)                 */
    FEEC_CUDA_ERROR = 7,     /* a CUDA runtime call failed                                     */
    FEEC_NO_DEVICE = 8       /* no usable GPU                                                  */
} feec_status;

/* Method selectors for feec_system_solve. */
enum {
    FEEC_METHOD_CG = 0,        /* ConjugateGradientSolverCSR          (sparsesolver.cpp:26-201)   */
    FEEC_METHOD_SSOR = 1,      /* ConjugateGradientSolverCSR_SSOR     (sparsesolver.cpp:446-724)  */
    FEEC_METHOD_RAINBOW = 2,   /* ConjugateGradientSolverCSR_Rainbow  (sparsesolver.cpp:1002-1335) */
    FEEC_METHOD_SSOR_EISENSTAT = 3,    /* ConjugateGradientSolverCSR_SSOR_Eisenstat (sparsesolver.cpp:726-995);
                                          needs feec_system_set_ssor; FEEC_MODE_REFERENCE only     */
    FEEC_METHOD_RAINBOW_EISENSTAT = 4, /* ConjugateGradientSolverCSR_Eisenstat_Rainbow (sparsesolver.cpp:1338-1645);
                                          needs feec_system_set_rainbow; FEEC_MODE_REFERENCE only  */
    FEEC_METHOD_DIAGONAL = 5           /* ConjugateGradientSolverCSR_DiagonalPreconditioner (sparsesolver.cpp:221-416);
                                          needs feec_system_set_diagonal_precon; REFERENCE only    */
};

/* Arithmetic / stopping modes for feec_system_solve. */
enum {
    FEEC_MODE_REFERENCE = 0,   /* FP64, the reference's stopping rule: sqrt(r.r) (CG) or |z.r|
                                  (PCG) below max(precision*||b||, 2^-26), cap N iterations  */
    FEEC_MODE_FP64 = 1,        /* FP64, stop on the true relative residual ||b-Ax||/||b||
                                  <= precision, no absolute floor                            */
    FEEC_MODE_MIXED = 2        /* FP32 inner PCG with compensated dots inside an FP64
                                  defect-correction loop; stop on the FP64 true relative
                                  residual <= precision                                      */
};

typedef struct feec_solve_info {
    int status;              /* feec_status of the solve                                   */
    int iterations;          /* K as the reference returns it (inner iterations in MIXED)  */
    int outer_iterations;    /* FP64 defect-correction steps (MIXED), else 1               */
    int num_colors;          /* colors / levels used by the preconditioner sweeps          */
    double tolerance;        /* max(precision*||b||, 2^-26) in REFERENCE mode, else precision */
    double final_norm;       /* sqrt of the quantity the stopping rule tested               */
    double true_relres;      /* ||b - A x|| / ||b|| in FP64 after the solve (-1 if skipped) */
    double device_ms;        /* time of the solve on the device (CUDA events)              */
    double total_ms;         /* wall time of the call including copies                     */
    int grid_blocks;         /* persistent grid size used                                  */
    int lanes_per_row;       /* CSR lanes per row used by the SpMV and sweeps              */
    int fp64_fallback;       /* MIXED: 1 if FP32 inner solves stagnated (operator too       */
                             /* ill-conditioned for FP32) and the solve finished in FP64    */
    int inner_fp64;          /* MIXED: 1 if the inner iterations ran in FP64: a reusable     */
                             /* batch measured them faster (feec_batch_create), or a system  */
                             /* solving on the whole GPU did (its first solve runs FP32,     */
                             /* its second FP64, later ones the faster per decade of fall)   */
    double error_estimate;   /* MIXED: estimated ||x - x*|| / ||x*|| from the measured      */
                             /* error-to-residual amplification of the outer corrections;   */
                             /* the solve keeps it <= 10 x precision; -1 if not estimated   */
} feec_solve_info;

/* ---------------------------------------------------------------------------
 * Drop-in entry points (host pointers). Arguments and return semantics follow
 * solver/sparsesolver.hpp; the iteration count is returned in info->iterations.
 * ------------------------------------------------------------------------- */

/* Replaces ConjugateGradientSolverCSR, solver/sparsesolver.hpp:11-19 (sparsesolver.cpp:26-201). */
int feec_cg_csr(int N, double* x, const double* b,
                const int* A, const int* C, const double* V,
                double* residual, double precision, int print_modulo,
                feec_solve_info* info);

/* Replaces ConjugateGradientSolverCSR_DiagonalPreconditioner, solver/sparsesolver.hpp:21-31
 * (sparsesolver.cpp:221-416): CG preconditioned by z = precon * r (rows with precon == 0 are
 * skipped, as in the reference). */
int feec_cg_csr_diagonal_precon(int N, double* x, const double* b,
                                const int* A, const int* C, const double* V,
                                double* residual, double precision, int print_modulo,
                                const double* precon, feec_solve_info* info);

/* Replaces ConjugateGradientSolverCSR_SSOR, solver/sparsesolver.hpp:33-43 (sparsesolver.cpp:446-724). */
int feec_cg_csr_ssor(int N, double* x, const double* b,
                     const int* A, const int* C, const double* V,
                     double* residual, double precision, int print_modulo,
                     const double* diagonal, double omega,
                     feec_solve_info* info);

/* Replaces ConjugateGradientSolverCSR_Rainbow, solver/sparsesolver.hpp:59-70 (sparsesolver.cpp:1002-1335). */
int feec_cg_csr_rainbow(int N, double* x, const double* b,
                        const int* A, const int* C, const double* V,
                        double* residual, double precision, int print_modulo,
                        const double* diagonal, double omega,
                        int num_colors, const int* F, const int* B, const int* R,
                        feec_solve_info* info);

/* Replaces ConjugateGradientSolverCSR_SSOR_Eisenstat, solver/sparsesolver.hpp:46-56
 * (sparsesolver.cpp:726-995). As in the reference, `residual` receives the residual of
 * the L-solved system the iteration works on. */
int feec_cg_csr_ssor_eisenstat(int N, double* x, const double* b,
                               const int* A, const int* C, const double* V,
                               double* residual, double precision, int print_modulo,
                               const double* diagonal, double omega,
                               feec_solve_info* info);

/* Replaces ConjugateGradientSolverCSR_Eisenstat_Rainbow, solver/sparsesolver.hpp:73-84
 * (sparsesolver.cpp:1338-1645). */
int feec_cg_csr_eisenstat_rainbow(int N, double* x, const double* b,
                                  const int* A, const int* C, const double* V,
                                  double* residual, double precision, int print_modulo,
                                  const double* diagonal, double omega,
                                  int num_colors, const int* F, const int* B, const int* R,
                                  feec_solve_info* info);

/* Replaces ConjugateResidualSolverCSR, solver/sparsesolver.hpp:89-97 (sparsesolver.cpp:1687-1915):
 * stops when |r.A r| < tolerance^2, the reference's rule; `residual` receives the recursive
 * residual. */
int feec_cr_csr(int N, double* x, const double* b,
                const int* A, const int* C, const double* V,
                double* residual, double precision, int print_modulo,
                feec_solve_info* info);

/* Replaces ConjugateResidualSolverCSR_textbook, solver/sparsesolver.hpp:99-107
 * (sparsesolver.cpp:1918-2156); the same arithmetic as ConjugateResidualSolverCSR. */
int feec_cr_csr_textbook(int N, double* x, const double* b,
                         const int* A, const int* C, const double* V,
                         double* residual, double precision, int print_modulo,
                         feec_solve_info* info);

/* Replaces MINRESCSR, solver/sparsesolver.hpp:112-120 (sparsesolver.cpp:2159-2425): stops
 * when |eta| < tolerance; `residual` receives b - A x. */
int feec_minres_csr(int N, double* x, const double* b,
                    const int* A, const int* C, const double* V,
                    double* residual, double precision, int print_modulo,
                    feec_solve_info* info);

/* Replaces ChebyshevIteration_DiagonalPreconditioner, solver/sparsesolver.hpp:127-139
 * (sparsesolver.cpp:2428-2590): z = precon * r, spectral bounds [lower, upper] of the
 * preconditioned operator; stops when ||r|| < tolerance. As in the reference, x receives
 * the iterate before the last one computed. */
int feec_chebyshev_diag(int N, double* x, const double* b,
                        const int* A, const int* C, const double* V,
                        double* residual, double precision, int print_modulo,
                        const double* precon, double lower, double upper,
                        feec_solve_info* info);

/* Hodge conjugate residual solvers, solver/systemsparsesolver.hpp:10-72
 * (systemsparsesolver.cpp:18-1120): conjugate residuals on M = B A^-1 Bt + C with
 * A (L x L), B (N x L), Bt (L x N), C (N x N), x, b, residual of N entries; A^-1 applied by
 * an inner CG on A to inner_precision (feec_hodge_cr_csr_diagonal: CG with precon
 * 1/diag(A); feec_hodge_cr_csr_ssor and feec_hodge_cr_csr: SSOR-PCG with omega = 1;
 * feec_hodge_cr_csr_textbook: plain CG). The outer stopping rule is the reference's
 * (|Mr.r| < tolerance^2). info->iterations is the outer K; info->outer_iterations holds the
 * total count of inner iterations. inner_print_modulo is accepted and not used (inner
 * solves are silent). */
#define FEEC_HODGE_PARAMS                                                                              \
    int N, int L, double* x, const double* b,                                                          \
    const int* Arows, const int* Acolumns, const double* Avalues,                                      \
    const int* Brows, const int* Bcolumns, const double* Bvalues,                                      \
    const int* Btrows, const int* Btcolumns, const double* Btvalues,                                   \
    const int* Crows, const int* Ccolumns, const double* Cvalues,                                      \
    double* residual, double precision, int print_modulo,                                              \
    double inner_precision, int inner_print_modulo, feec_solve_info* info
int feec_hodge_cr_csr(FEEC_HODGE_PARAMS);            /* HodgeConjugateResidualSolverCSR          (:18-50)    */
int feec_hodge_cr_csr_diagonal(FEEC_HODGE_PARAMS);   /* HodgeConjugateResidualSolverCSR_diagonal (:52-424)   */
int feec_hodge_cr_csr_ssor(FEEC_HODGE_PARAMS);       /* HodgeConjugateResidualSolverCSR_SSOR     (:426-796)  */
int feec_hodge_cr_csr_textbook(FEEC_HODGE_PARAMS);   /* HodgeConjugateResidualSolverCSR_textbook (:798-1120) */

/* Replaces HodgeHerzogSoodhalterMethod, solver/systemsparsesolver.hpp:74-95
 * (systemsparsesolver.cpp:1122-1575): preconditioned MINRES on [[-A, Bt], [B, C]] [x_A; x_C] =
 * [b_A; b_C] (A: dim_A x dim_A, Bt: dim_A x dim_C, B: dim_C x dim_A, C: dim_C x dim_C) with the
 * block preconditioner diag(PA, PC) applied by inner CG solves to inner_precision; a block
 * whose three arrays are not all given is skipped, as in the reference. Returns the
 * reference's status through info; info->iterations is its iteration count and
 * info->outer_iterations the total of inner iterations. */
int feec_hodge_herzog_soodhalter(int dimension_A, int dimension_C, double* x_A, double* x_C,
                                 const double* b_A, const double* b_C,
                                 const int* Arows, const int* Acolumns, const double* Avalues,
                                 const int* Brows, const int* Bcolumns, const double* Bvalues,
                                 const int* Btrows, const int* Btcolumns, const double* Btvalues,
                                 const int* Crows, const int* Ccolumns, const double* Cvalues,
                                 double precision, int print_modulo,
                                 const int* PArows, const int* PAcolumns, const double* PAvalues,
                                 const int* PCrows, const int* PCcolumns, const double* PCvalues,
                                 double inner_precision, int inner_print_modulo, feec_solve_info* info);

/* Replaces MatrixCSR::apply(dest, src, scaling), sparse/matcsr.cpp:216-244:
 * dest = scaling * A * src (rows x cols matrix, host pointers). */
int feec_csr_apply(int rows, int cols, const int* A, const int* C, const double* V,
                   const double* src, double* dest, double scaling);

/* Replaces MatrixCSR::getDiagonal, sparse/matcsr.cpp:266-286 (host pointers). */
int feec_csr_diagonal(int N, const int* A, const int* C, const double* V, double* diagonal);

/* CSR algebra on the GPU (host pointers; inputs checked on the host first, FEEC_BADARG on
 * row pointers that are not monotone from 0 or columns out of range). Results are the
 * reference's bit for bit: entries laid out in the reference's order, rows compressed
 * by the reference's exchange sort (sparse/matcsr.cpp:585-688, sort_and_compress_csrdata_reduced),
 * entries that sum to zero dropped. *nnz receives the final entry count.
 *
 * Replaces MatrixCSRAddition(mat1, mat2, s1, s2), sparse/matcsr.cpp:707-765:
 * s1 * (A1,C1,V1) + s2 * (A2,C2,V2), both rows x cols. A has rows+1 entries; C and V
 * need A1[rows] + A2[rows] entries of room. */
int feec_csr_add(int rows, int cols, const int* A1, const int* C1, const double* V1,
                 const int* A2, const int* C2, const double* V2, double s1, double s2,
                 int* A, int* C, double* V, int* nnz);

/* Entries of (rows x inner) * (inner x cols) before compression, sparse/matcsr.cpp:776-796:
 * the room C and V need for feec_csr_multiply. */
int feec_csr_multiply_size(int rows, int inner, const int* A1, const int* C1, const int* A2,
                           long long* size);

/* Replaces MatrixCSRMultiplication(mat1, mat2), sparse/matcsr.cpp:767-849. FEEC_BADARG when
 * the uncompressed product exceeds INT_MAX entries (the reference's int offsets). */
int feec_csr_multiply(int rows, int inner, int cols, const int* A1, const int* C1, const double* V1,
                      const int* A2, const int* C2, const double* V2,
                      int* A, int* C, double* V, int* nnz);

/* Replaces MatrixCSR::getTranspose, sparse/matcsr.cpp:291-350: (A,C,V) rows x cols to
 * (B,D,W) cols x rows. B has cols+1 entries; D and W need A[rows] entries of room. */
int feec_csr_transpose(int rows, int cols, const int* A, const int* C, const double* V,
                       int* B, int* D, double* W, int* nnz);

/* Replaces MatrixCSR(const SparseMatrix&), sparse/matcsr.cpp:43-89 with
 * SparseMatrix::sortandcompressentries, sparse/sparsematrix.cpp:405-458: `count` COO
 * entries (row r[i], column c[i], value v[i]) to CSR; zero values dropped, entries at the
 * same position summed in input order (the reference's std::sort leaves that order
 * unspecified, so sums of duplicates can differ from it in the last bit). A has rows+1
 * entries; C and V need `count` entries of room. */
int feec_coo_to_csr(int rows, int cols, long long count, const int* r, const int* c, const double* v,
                    int* A, int* C, double* V, int* nnz);

/* Upper bound on the entries of a COO product (left lrows x inner with ln entries, right
 * inner x rcols with rn entries): for every k, left entries in column k times right entries
 * in row k (sparse/sparsematrix.cpp:622-660 counts the same after compressing). */
int feec_coo_multiply_size(int inner, long long ln, const int* lc, long long rn, const int* rr,
                           long long* size);

/* Replaces SparseMatrixMultiplication(left, right), sparse/sparsematrix.cpp:609-722: both
 * operands compressed (zeros dropped, equal positions summed in input order), every product
 * L(i,k) R(k,j), zero products dropped, equal positions summed in k order; the result
 * row-wise sorted in out_r/out_c/out_v (room: feec_coo_multiply_size), *count entries. The
 * reference's std::sort leaves the summation order of equal positions unspecified, so
 * entries with several products can differ from it in rounding (the structure and entries
 * with one product are identical). */
int feec_coo_multiply(int lrows, int inner, int rcols,
                      long long ln, const int* lr, const int* lc, const double* lv,
                      long long rn, const int* rr, const int* rc, const double* rv,
                      int* out_r, int* out_c, double* out_v, long long* count);

/* Replaces Rainbow::Rainbow(mat, do_shuffle = false), sparse/rainbow.cpp:14-130.
 * F[N], B[N+1] (num_colors+1 entries used), R[N], host pointers; bit-identical
 * to the reference's greedy coloring. */
int feec_rainbow(int N, const int* A, const int* C, int* num_colors, int* F, int* B, int* R);

/* Replaces MatrixCSR::check's structural invariants, sparse/matcsr.cpp:178-194:
 * FEEC_OK if A is non-decreasing from 0 to nnz, 0 <= C < cols and V finite. */
int feec_csr_check(int rows, int cols, const int* A, const int* C, const double* V);

/* ---------------------------------------------------------------------------
 * Device-resident systems (device pointers, explicit stream).
 * ------------------------------------------------------------------------- */

typedef struct feec_system feec_system;

/* Uploads (host_ptrs != 0) or adopts a copy of (host_ptrs == 0, device pointers)
 * an N x N CSR matrix. `stream` is a cudaStream_t; NULL is CUDA's default stream
 * (stream 0). It becomes the system's stream; every feec_system_* call below runs on
 * its own `stream` argument if that is not NULL, else on the system's stream. */
int feec_system_create(feec_system** sys, int N, const int* A, const int* C, const double* V,
                       int host_ptrs, void* stream);

/* Prepares the multicolor SSOR layout from a Rainbow coloring (F, B, R as in
 * sparse/rainbow.hpp:22-30) and the diagonal. Pointers are host pointers if
 * host_ptrs != 0, else device pointers. */
int feec_system_set_rainbow(feec_system* sys, const double* diagonal, double omega,
                            int num_colors, const int* F, const int* B, const int* R, int host_ptrs);

/* Sets the diagonal preconditioner of FEEC_METHOD_DIAGONAL (N values; host pointer if
 * host_ptrs != 0, else device pointer). */
int feec_system_set_diagonal_precon(feec_system* sys, const double* precon, int host_ptrs);

/* Prepares the lexicographic SSOR layout (level-scheduled triangular sweeps). */
int feec_system_set_ssor(feec_system* sys, const double* diagonal, double omega, int host_ptrs);

/* Solves A x = b on the device. x (in/out, initial guess), b and residual are
 * device pointers of N doubles (residual may be NULL). max_iter <= 0 means N.
 * FEEC_MODE_MIXED (here and in the batched and serving entry points below): when an
 * FP32 inner solve gains less than half the digits it was asked for (condition
 * number times FP32 roundoff near 1e-2 or above), the solve continues in FP64 from
 * its current iterate with a fresh budget of max_iter iterations, and
 * info->fp64_fallback is 1. */
int feec_system_solve(feec_system* sys, int method, int mode, double* x, const double* b,
                      double* residual, double precision, int max_iter,
                      feec_solve_info* info, void* stream);

/* Batched solves of one system with many right-hand sides (FEEC_MODE_MIXED or
 * FEEC_MODE_FP64; FEEC_METHOD_CG or FEEC_METHOD_RAINBOW): X and B are device
 * arrays of nrhs columns of N doubles (column j at X + j*N). One thread block
 * advances rhs_per_team columns (1, 2, 4 or 8 in FP32 / MIXED; 1 or 2 in FP64;
 * 0 = automatic) through a complete
 * solve; blocks take columns from a queue until none are left. infos (host,
 * nrhs entries, may be NULL) receives each column's result. */
int feec_system_solve_batch(feec_system* sys, int method, int mode, int nrhs, double* X, const double* B,
                            double precision, int max_iter, int rhs_per_team,
                            feec_solve_info* infos, void* stream);

/* Autotuner of the batched engine: times short trials of every launch candidate
 * (right-hand sides per team 1/2/4/8; a one-block team of 128..1024 threads, or —
 * when nrhs_hint leaves fewer work items than the GPU holds one-block teams — a
 * cluster team of 2/4/8/16 blocks) on this system and caches the fastest, which
 * feec_system_solve_batch then uses whenever rhs_per_team is 0. nrhs_hint is the
 * batch size to tune for (0 = fill the GPU). Outputs may be NULL; *team_blocks is
 * 1 for a one-block team. */
int feec_system_tune_batch(feec_system* sys, int method, int mode, int nrhs_hint,
                           int* rhs_per_team, int* team_threads, int* team_blocks,
                           double* rhs_iters_per_s);

/* Sets the batched launch configuration used when rhs_per_team is 0, as the
 * autotuner would (rhs_per_team 0 clears it). team_blocks 1: one-block teams of
 * team_threads (128/256/512/1024) threads; 2..16 (power of two): cluster teams
 * of that many 512-thread blocks (team_threads ignored). */
int feec_system_set_batch_config(feec_system* sys, int method, int mode, int rhs_per_team,
                                 int team_threads, int team_blocks);

/* Batched solves of many systems, one right-hand side each (device pointers
 * x[i], b[i] of systems[i]->N doubles; host arrays of pointers). Systems are
 * processed largest first, one thread block per system. For
 * FEEC_METHOD_RAINBOW every system must have been prepared with
 * feec_system_set_rainbow. */
int feec_solve_many(int nsys, feec_system* const* systems, int method, int mode,
                    double* const* x, const double* const* b, double precision, int max_iter,
                    feec_solve_info* infos, void* stream);

/* A reusable batch over many systems (one right-hand side each, device pointers
 * x[i], b[i] that stay valid for the batch's lifetime; x holds the initial guess
 * on every run). Everything is set up once and the launch sequence is captured in
 * a CUDA graph; feec_batch_run replays it and fills infos[i] (host, nsys entries,
 * may be NULL) and *device_ms. team_threads 0 = 256. In FEEC_MODE_MIXED the create
 * call solves the batch once with FP32 and once with FP64 inner iterations (x is
 * restored afterwards) and keeps the faster; infos[i].inner_fp64 reports it. */
typedef struct feec_batch feec_batch;
int feec_batch_create(feec_batch** batch, int nsys, feec_system* const* systems, int method, int mode,
                      double* const* x, const double* const* b, double precision, int max_iter,
                      int team_threads, void* stream);
int feec_batch_run(feec_batch* batch, feec_solve_info* infos, double* device_ms);
/* feec_batch_run in two halves, so that one host thread can overlap other work (the
 * next batch's uploads, the last batch's downloads on its own streams) with a replay:
 * feec_batch_launch enqueues the replay after the work already on the caller's stream
 * and returns at once; feec_batch_finish waits for it and fills infos and *device_ms
 * as feec_batch_run does. x and b of the batch must not be touched in between. A
 * second launch before the finish, or a finish without a launch, is FEEC_BADARG.
 * Several batches (over separate x, b) may be in flight at the same time. */
int feec_batch_launch(feec_batch* batch);
int feec_batch_finish(feec_batch* batch, feec_solve_info* infos, double* device_ms);
int feec_batch_destroy(feec_batch* batch);

/* y = scaling * A * x with device pointers (MatrixCSR::apply on a resident matrix),
 * over a cached SELL-32 copy of the matrix, one thread per row. */
int feec_system_apply(feec_system* sys, const double* x, double* y, double scaling, void* stream);

/* The same product on the FP32 copy of the values (x, y float). */
int feec_system_apply_f32(feec_system* sys, const float* x, float* y, float scaling, void* stream);

/* Launch-shape override for the persistent solvers (used by the autotuner):
 * blocks = co-resident grid size, lanes = CSR lanes per row (power of two <= 32);
 * 0 restores the automatic choice. Sizes beyond the co-resident limit are clamped. */
int feec_system_set_launch(feec_system* sys, int blocks, int lanes);

/* Bytes of device memory held by the system. */
int feec_system_memory(const feec_system* sys, size_t* bytes);

int feec_system_destroy(feec_system* sys);

/* No counterpart in the reference. Plain CG (reference stopping rule) for callers
 * that cannot allocate device memory during a solve: every pointer is a device
 * pointer the caller owns, and the solver's scratch is a fixed 16 MiB file-scope
 * device array of this library instead of an allocation. At most 1,048,576 rows
 * (larger N returns FEEC_BADARG). All calls share that array: calls that overlap
 * on the GPU race and must be serialised by the caller. The first call on a
 * device looks up the array's address; make it before any stream capture.
 * max_iter <= 0 means N; `stream` is a cudaStream_t (NULL = legacy default).
 * Every return, early ones included, also stores its code in info->status. */
int feec_cg_csr_noalloc(int N, double* x, const double* b,
                        const int* A, const int* C, const double* V,
                        double* residual, double precision, int max_iter,
                        feec_solve_info* info, void* stream);

/* ---------------------------------------------------------------------------
 * Serving loop with continuous batching. A server owns `slots` worker slots; each
 * submitted request (one SPD solve) waits in a FIFO queue until a slot is free and
 * the device memory budget has room for its estimated footprint, then is set up
 * (matrix upload, Rainbow coloring, multicolor SSOR layout) and solved as one
 * thread-block cluster on the slot's own stream, overlapping with the requests in
 * the other slots. method: FEEC_METHOD_RAINBOW or FEEC_METHOD_CG; mode:
 * FEEC_MODE_MIXED or FEEC_MODE_FP64 (true FP64 relative residual <= precision).
 * ------------------------------------------------------------------------- */

typedef struct feec_server feec_server;

typedef struct feec_request_result {
    long long id;
    int n;                   /* unknowns                                            */
    int status;              /* feec_status of the solve                            */
    int iterations;          /* inner iterations                                    */
    int outer_iterations;    /* FP64 defect-correction steps                        */
    int cluster_blocks;      /* thread blocks of the cluster that solved it         */
    int fp64_fallback;       /* 1 if mixed precision stagnated and FP64 finished it */
    double true_relres;      /* ||b - A x|| / ||b|| in FP64 at the end               */
    double t_submit_ms;      /* host steady-clock times since the server started    */
    double t_start_ms;       /* solve launched (after admission and set-up)         */
    double t_end_ms;         /* solution copied back                                */
    double error_estimate;   /* mixed: estimated relative error of x (-1: none)     */
} feec_request_result;

int feec_server_create(feec_server** srv, size_t hbm_budget_bytes, int slots, int method, int mode);

/* Queues one request. Host arrays A, C, V (N x N CSR), b and the output x must stay
 * valid until the request is reported by feec_server_poll. *id identifies it.
 * FEEC_OOM if its estimated footprint exceeds the whole budget. */
int feec_server_submit(feec_server* srv, int N, const int* A, const int* C, const double* V,
                       const double* b, double* x, double precision, long long* id);

/* Resident operators, for streams of right-hand sides on the same matrices: the matrix
 * is uploaded and prepared once (coloring, layouts) in the calling thread, its estimated
 * footprint reserved in the budget (FEEC_OOM if it does not fit beside what runs now),
 * and *op identifies it. Requests submitted against it carry only their right-hand side
 * and solution (host b, x valid until reported) and share the prepared matrix; a request
 * on the whole-GPU solver also keeps the system's measured mixed-precision choice from
 * one request to the next. An operator can be removed once no request on it is queued or
 * running (FEEC_BADARG otherwise). */
int feec_server_add_operator(feec_server* srv, int N, const int* A, const int* C, const double* V, int* op);
int feec_server_submit_rhs(feec_server* srv, int op, const double* b, double* x, double precision, long long* id);
int feec_server_remove_operator(feec_server* srv, int op);

/* Moves up to max_out finished requests into out; *nout receives their number. */
int feec_server_poll(feec_server* srv, feec_request_result* out, int max_out, int* nout);

/* Blocks until every submitted request has finished (FEEC_TIMEOUT after timeout_s). */
int feec_server_wait(feec_server* srv, double timeout_s);

int feec_server_stats(feec_server* srv, size_t* bytes_in_use, size_t* peak_bytes, int* inflight, long long* queued);

/* Finishes the queued requests, then stops the slots. */
int feec_server_destroy(feec_server* srv);

/* ---------------------------------------------------------------------------
 * Library information.
 * ------------------------------------------------------------------------- */

/* Number of kernels this library launched since load (all devices). */
unsigned long long feec_kernel_launches(void);

/* Human-readable name of a status code. */
const char* feec_status_string(int status);

/* Self-test of the bounded device waits (no counterpart in the reference): runs a
 * kernel whose single wait is never satisfied, with a limit of limit_s seconds (at
 * most 10). The wait gives up as a solver's grid barrier does; *status receives the
 * status the kernel recorded (FEEC_TIMEOUT), *site the wait site, *elapsed_ms the host
 * time of the call. Returns FEEC_OK when the GPU answered normally afterwards. */
int feec_selftest_wait_timeout(double limit_s, int* status, int* site, double* elapsed_ms);

#ifdef __cplusplus
}
#endif

#endif /* FEEC_GPU_H */
