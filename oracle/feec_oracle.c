/*
 * ORACLE — test infrastructure, not product code.
 *
 * A plain-C restatement of the FEEC++ reference algorithms on the sparse CSR
 * Krylov path and the CSR algebra and block solvers around it, used only to compare
 * results against by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
 * reference legs. Nothing in the product library
 * links, loads or calls this file.
 *
 * Every function follows the cited reference lines statement by statement,
 * including loop order and accumulation order, so that at one OpenMP thread
 * its outputs are bit-identical to the reference's on the same inputs (pinned
 * by tests/test_oracle.py against fixtures written by the reference itself).
 * Build with -ffp-contract=off so that no fused multiply-add changes rounding.
 *
 * OpenMP is used exactly where the reference uses `parallel for`. The plain CG
 * direction update (solver/sparsesolver.cpp:179-183) is `omp parallel` without
 * `for` in the reference, a race that stops convergence with more than one
 * thread; the restatement runs that loop serially, which is what the reference
 * computes at one thread.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* base/base.hpp:123, 127-128: machine_epsilon = 2^-52, desired_precision = sqrt(machine_epsilon) */
static const double ORACLE_MACHINE_EPSILON = 2.220446049250313080847263336181640625e-16;
static const double ORACLE_DESIRED_PRECISION = 1.490116119384765625e-08;

static double dmax(double a, double b) { return a > b ? a : b; }

/* sparse/matcsr.cpp:216-244: dest = 0; dest[i] += scaling * V[j] * src[C[j]] */
void oracle_csr_apply(int N, const int* A, const int* C, const double* V,
                      const double* src, double* dest, double scaling)
{
    for (int i = 0; i < N; i++) dest[i] = 0.0;
    #pragma omp parallel for
    for (int i = 0; i < N; i++)
        for (int j = A[i]; j < A[i + 1]; j++)
            dest[i] += scaling * V[j] * src[C[j]];
}

/* sparse/matcsr.cpp:266-286: sum of the stored entries with C == row */
void oracle_csr_diagonal(int N, const int* A, const int* C, const double* V, double* diag)
{
    #pragma omp parallel for
    for (int r = 0; r < N; r++) {
        diag[r] = 0.0;
        for (int i = A[r]; i < A[r + 1]; i++)
            if (C[i] == r) diag[r] += V[i];
    }
}

/* sparse/rainbow.cpp:14-130 with do_shuffle = false. F[N], B[N+1] (only
 * num_colors+1 used), R[N]. Returns num_colors, or -1 on an invalid result. */
int oracle_rainbow(int N, const int* A, const int* C, int* F, int* B, int* R)
{
    int num_colors = 1;                                       /* :35 */
    for (int r = 0; r < N; r++) F[r] = 0;                     /* :46 */
    for (int r = 0; r < N; r++) {                             /* :48-75, painting order = identity */
    again:
        for (int c = A[r]; c < A[r + 1]; c++) {
            int j = C[c];
            if (j == r) continue;
            if (F[j] == F[r]) { F[r]++; goto again; }
        }
        if (F[r] == num_colors) num_colors++;
    }
    int* counter = (int*)calloc((size_t)num_colors, sizeof(int));   /* :81-85 */
    if (!counter) return -1;
    for (int r = 0; r < N; r++) counter[F[r]]++;
    B[0] = 0;                                                 /* :91-93 */
    for (int c = 1; c < num_colors + 1; c++) B[c] = counter[c - 1];
    for (int c = 1; c < num_colors + 1; c++) B[c] += B[c - 1];
    for (int r = 0; r < N; r++) R[r] = -1;                    /* :101-117: filled from the top of each color */
    for (int r = 0; r < N; r++) {
        int color = F[r];
        counter[color]--;
        R[B[color] + counter[color]] = r;
    }
    free(counter);
    return num_colors;
}

/* solver/sparsesolver.cpp:26-201, unpreconditioned CG; returns K */
int oracle_cg(int N, double* x, const double* b, const int* A, const int* C, const double* V,
              double* residual, double precision, int print_modulo)
{
    (void)print_modulo;
    double tolerance = 0.0;                                   /* :45-48 */
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = precision * sqrt(tolerance);
    tolerance = dmax(tolerance, ORACLE_DESIRED_PRECISION);

    double* direction = (double*)malloc(sizeof(double) * (size_t)N);   /* :62-63 */
    double* auxiliary = (double*)malloc(sizeof(double) * (size_t)N);
    if (!direction || !auxiliary) { free(direction); free(auxiliary); return -1; }
    for (int i = 0; i < N; i++) direction[i] = auxiliary[i] = NAN;

    double r_r = NAN;
    int K = 0;
    while (K < N) {                                           /* :74 */
        if (K == 0) {                                         /* :76-104 */
            r_r = 0.0;
            #pragma omp parallel for reduction(+:r_r)
            for (int c = 0; c < N; c++) {
                residual[c] = b[c];
                for (int d = A[c]; d < A[c + 1]; d++) residual[c] -= V[d] * x[C[d]];
                direction[c] = residual[c];
                r_r += residual[c] * residual[c];
            }
        }
        if (fabs(r_r) < tolerance * tolerance) break;        /* :116-119 */

        double d_Ad = 0.0;                                    /* :126-139 */
        #pragma omp parallel for reduction(+:d_Ad)
        for (int c = 0; c < N; c++) {
            auxiliary[c] = 0.0;
            for (int d = A[c]; d < A[c + 1]; d++) auxiliary[c] += V[d] * direction[C[d]];
            d_Ad += direction[c] * auxiliary[c];
        }
        int numerator_bad = !isfinite(r_r) || r_r < 0.0;      /* :142-155 */
        int denominator_bad = !isfinite(d_Ad) || d_Ad < 0.0;
        int denominator_small = sqrt(fabs(d_Ad)) < ORACLE_MACHINE_EPSILON;
        if (numerator_bad || denominator_bad) break;
        if (denominator_small) break;

        double alpha = r_r / d_Ad;                            /* :158-173 */
        double r_r_new = 0.0;
        #pragma omp parallel for reduction(+:r_r_new)
        for (int c = 0; c < N; c++) {
            x[c] += alpha * direction[c];
            residual[c] -= alpha * auxiliary[c];
            r_r_new += residual[c] * residual[c];
        }
        double beta = r_r_new / r_r;                          /* :175-183 */
        r_r = r_r_new;
        for (int c = 0; c < N; c++) direction[c] = residual[c] + beta * direction[c];
        K++;
    }
    free(direction);
    free(auxiliary);
    return K;
}

static double* nan_vector(int N);

/* solver/sparsesolver.cpp:221-416, CG with a diagonal preconditioner z = precon * r;
 * returns K. The direction update (:386-395) is `omp parallel` without `for` in the
 * reference (a race with more than one thread); it runs serially here. */
int oracle_cg_diag(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                   double* residual, double precision, int print_modulo, const double* precon)
{
    (void)print_modulo;
    double tolerance = 0.0;                                   /* :243-246 */
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = precision * sqrt(tolerance);
    tolerance = dmax(tolerance, ORACLE_DESIRED_PRECISION);

    double* direction = nan_vector(N);                        /* :259-264 */
    double* zirconium = nan_vector(N);
    double* auxiliary = nan_vector(N);
    if (!direction || !zirconium || !auxiliary) {
        free(direction); free(zirconium); free(auxiliary); return -1;
    }
    double z_r = NAN;
    int K = 0;
    while (K < N) {
        if (K == 0) {                                         /* :283-302 */
            z_r = 0.0;
            #pragma omp parallel for reduction(+:z_r)
            for (int c = 0; c < N; c++) {
                if (precon[c] == 0.0) continue;
                residual[c] = b[c];
                for (int d = A[c]; d < A[c + 1]; d++) residual[c] -= V[d] * x[C[d]];
                zirconium[c] = precon[c] * residual[c];
                direction[c] = zirconium[c];
                z_r += zirconium[c] * residual[c];
            }
        }
        if (fabs(z_r) < tolerance * tolerance) break;        /* :318-321 */

        double d_Ad = 0.0;                                    /* :330-345 */
        #pragma omp parallel for reduction(+:d_Ad)
        for (int c = 0; c < N; c++) {
            if (precon[c] == 0.0) continue;
            auxiliary[c] = 0.0;
            for (int d = A[c]; d < A[c + 1]; d++) auxiliary[c] += V[d] * direction[C[d]];
            d_Ad += direction[c] * auxiliary[c];
        }
        int numerator_bad = !isfinite(z_r) || z_r < 0.0;      /* :348-363 */
        int denominator_bad = !isfinite(d_Ad) || d_Ad < 0.0;
        int denominator_small = sqrt(fabs(d_Ad)) < ORACLE_MACHINE_EPSILON;
        if (numerator_bad || denominator_bad) break;
        if (denominator_small) break;

        const double alpha = z_r / d_Ad;                      /* :366-384 */
        double z_r_new = 0.0;
        #pragma omp parallel for reduction(+:z_r_new)
        for (int c = 0; c < N; c++) {
            if (precon[c] == 0.0) continue;
            x[c] += alpha * direction[c];
            residual[c] -= alpha * auxiliary[c];
            zirconium[c] = precon[c] * residual[c];
            z_r_new += zirconium[c] * residual[c];
        }
        const double beta = z_r_new / z_r;                    /* :386-397 */
        z_r = z_r_new;
        for (int c = 0; c < N; c++) {
            if (precon[c] == 0.0) continue;
            direction[c] = zirconium[c] + beta * direction[c];
        }
        K++;
    }
    free(direction); free(zirconium); free(auxiliary);
    return K;
}

/* solver/sparsesolver.cpp:446-724, SSOR-preconditioned CG in index order; returns K */
int oracle_cg_ssor(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                   double* residual, double precision, int print_modulo,
                   const double* diagonal, double omega)
{
    (void)print_modulo;
    double tolerance = 0.0;                                   /* :463-466 */
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = precision * sqrt(tolerance);
    tolerance = dmax(tolerance, ORACLE_DESIRED_PRECISION);

    double* direction = (double*)calloc((size_t)N, sizeof(double));     /* :479-490 */
    double* zirconium = (double*)calloc((size_t)N, sizeof(double));
    double* auxiliary = (double*)calloc((size_t)N, sizeof(double));
    double* mittlerer = (double*)calloc((size_t)N, sizeof(double));
    if (!direction || !zirconium || !auxiliary || !mittlerer) {
        free(direction); free(zirconium); free(auxiliary); free(mittlerer); return -1;
    }
    double z_r = NAN;
    int K = 0;
    while (K < N) {
        if (K == 0) {                                         /* :506-588 */
            #pragma omp parallel for
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                residual[c] = b[c];
                for (int d = A[c]; d < A[c + 1]; d++) residual[c] -= V[d] * x[C[d]];
            }
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                double aux = residual[c];
                for (int d = A[c]; d < A[c + 1]; d++)
                    if (C[d] < c) aux -= V[d] * mittlerer[C[d]];
                mittlerer[c] = aux * omega / diagonal[c];
            }
            #pragma omp parallel for
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                mittlerer[c] *= diagonal[c];
                mittlerer[c] *= (2.0 - omega) / omega;
            }
            for (int c = N - 1; c >= 0; c--) {
                if (diagonal[c] == 0.0) continue;
                double aux = mittlerer[c];
                for (int d = A[c]; d < A[c + 1]; d++)
                    if (C[d] > c) aux -= V[d] * zirconium[C[d]];
                zirconium[c] = aux * omega / diagonal[c];
            }
            z_r = 0.0;
            #pragma omp parallel for reduction(+:z_r)
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                direction[c] = zirconium[c];
                z_r += zirconium[c] * residual[c];
            }
        }
        if (fabs(z_r) < tolerance * tolerance) break;        /* :601-604 */

        double d_Ad = 0.0;                                    /* :611-626 */
        #pragma omp parallel for reduction(+:d_Ad)
        for (int c = 0; c < N; c++) {
            auxiliary[c] = 0.0;
            if (diagonal[c] == 0.0) continue;
            for (int d = A[c]; d < A[c + 1]; d++) auxiliary[c] += V[d] * direction[C[d]];
            d_Ad += direction[c] * auxiliary[c];
        }
        int numerator_bad = !isfinite(z_r) || z_r < 0.0;
        int denominator_bad = !isfinite(d_Ad) || d_Ad < 0.0;
        int denominator_small = sqrt(fabs(d_Ad)) < ORACLE_MACHINE_EPSILON;
        if (numerator_bad || denominator_bad) break;
        if (denominator_small) break;

        const double alpha = z_r / d_Ad;                      /* :645-663 */
        for (int c = 0; c < N; c++) {
            if (diagonal[c] == 0.0) continue;
            x[c] += alpha * direction[c];
            residual[c] -= alpha * auxiliary[c];
            double aux = residual[c];
            for (int d = A[c]; d < A[c + 1]; d++)
                if (C[d] < c) aux -= V[d] * mittlerer[C[d]];
            mittlerer[c] = aux * omega / diagonal[c];
        }
        double z_r_new = 0.0;                                 /* :665-692 */
        for (int c = N - 1; c >= 0; c--) {
            if (diagonal[c] == 0.0) continue;
            mittlerer[c] *= diagonal[c];
            mittlerer[c] *= (2.0 - omega) / omega;
            double aux = mittlerer[c];
            for (int d = A[c]; d < A[c + 1]; d++)
                if (C[d] > c) aux -= V[d] * zirconium[C[d]];
            zirconium[c] = aux * omega / diagonal[c];
            z_r_new += zirconium[c] * residual[c];
        }
        const double beta = z_r_new / z_r;                    /* :694-709 */
        z_r = z_r_new;
        #pragma omp parallel for
        for (int c = 0; c < N; c++) {
            if (diagonal[c] == 0.0) continue;
            direction[c] = zirconium[c] + beta * direction[c];
        }
        K++;
    }
    free(direction); free(zirconium); free(auxiliary); free(mittlerer);
    return K;
}

/* solver/sparsesolver.cpp:1002-1335, multicolor ("Rainbow") SSOR-PCG; returns K */
int oracle_cg_rainbow(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                      double* residual, double precision, int print_modulo,
                      const double* diagonal, double omega,
                      int num_colors, const int* F, const int* B, const int* R)
{
    (void)print_modulo;
    double tolerance = 0.0;                                   /* :1030-1033 */
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = precision * sqrt(tolerance);
    tolerance = dmax(tolerance, ORACLE_DESIRED_PRECISION);

    double* direction = (double*)calloc((size_t)N, sizeof(double));     /* :1046-1057 */
    double* zirconium = (double*)calloc((size_t)N, sizeof(double));
    double* auxiliary = (double*)calloc((size_t)N, sizeof(double));
    double* mittlerer = (double*)calloc((size_t)N, sizeof(double));
    if (!direction || !zirconium || !auxiliary || !mittlerer) {
        free(direction); free(zirconium); free(auxiliary); free(mittlerer); return -1;
    }
    double z_r = NAN;
    int K = 0;
    while (K < N) {
        if (K == 0) {                                         /* :1072-1175 */
            #pragma omp parallel for
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                residual[c] = b[c];
                for (int d = A[c]; d < A[c + 1]; d++) residual[c] -= V[d] * x[C[d]];
            }
            for (int color = 0; color < num_colors; color++) {
                #pragma omp parallel for
                for (int i = B[color]; i < B[color + 1]; i++) {
                    int c = R[i];
                    if (diagonal[c] == 0.0) continue;
                    double aux = residual[c];
                    for (int d = A[c]; d < A[c + 1]; d++)
                        if (F[C[d]] < F[c]) aux -= V[d] * mittlerer[C[d]];
                    mittlerer[c] = aux * omega / diagonal[c];
                }
            }
            #pragma omp parallel for
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                mittlerer[c] *= diagonal[c];
                mittlerer[c] *= (2.0 - omega) / omega;
            }
            for (int color = num_colors - 1; color >= 0; color--) {
                #pragma omp parallel for
                for (int i = B[color]; i < B[color + 1]; i++) {
                    int c = R[i];
                    if (diagonal[c] == 0.0) continue;
                    double aux = mittlerer[c];
                    for (int d = A[c]; d < A[c + 1]; d++)
                        if (F[C[d]] > F[c]) aux -= V[d] * zirconium[C[d]];
                    zirconium[c] = aux * omega / diagonal[c];
                }
            }
            z_r = 0.0;
            #pragma omp parallel for reduction(+:z_r)
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                direction[c] = zirconium[c];
                z_r += zirconium[c] * residual[c];
            }
        }
        if (fabs(z_r) < tolerance * tolerance) break;        /* :1187-1190 */

        double d_Ad = 0.0;                                    /* :1197-1212 */
        #pragma omp parallel for reduction(+:d_Ad)
        for (int c = 0; c < N; c++) {
            auxiliary[c] = 0.0;
            if (diagonal[c] == 0.0) continue;
            for (int d = A[c]; d < A[c + 1]; d++) auxiliary[c] += V[d] * direction[C[d]];
            d_Ad += direction[c] * auxiliary[c];
        }
        int numerator_bad = !isfinite(z_r) || z_r < 0.0;
        int denominator_bad = !isfinite(d_Ad) || d_Ad < 0.0;
        int denominator_small = sqrt(fabs(d_Ad)) < ORACLE_MACHINE_EPSILON;
        if (numerator_bad || denominator_bad) break;
        if (denominator_small) break;

        const double alpha = z_r / d_Ad;                      /* :1230-1261 */
        for (int color = 0; color < num_colors; color++) {
            #pragma omp parallel for
            for (int i = B[color]; i < B[color + 1]; i++) {
                int c = R[i];
                if (diagonal[c] == 0.0) continue;
                x[c] += alpha * direction[c];
                residual[c] -= alpha * auxiliary[c];
                double aux = residual[c];
                for (int d = A[c]; d < A[c + 1]; d++)
                    if (F[C[d]] < F[c]) aux -= V[d] * mittlerer[C[d]];
                mittlerer[c] = aux * omega / diagonal[c];
            }
        }
        double z_r_new = 0.0;                                 /* :1263-1307 */
        for (int color = num_colors - 1; color >= 0; color--) {
            double z_r_new_local = 0.0;
            #pragma omp parallel for reduction(+:z_r_new_local)
            for (int i = B[color]; i < B[color + 1]; i++) {
                int c = R[i];
                if (diagonal[c] == 0.0) continue;
                mittlerer[c] *= diagonal[c];
                mittlerer[c] *= (2.0 - omega) / omega;
                double aux = mittlerer[c];
                for (int d = A[c]; d < A[c + 1]; d++)
                    if (F[C[d]] > F[c]) aux -= V[d] * zirconium[C[d]];
                zirconium[c] = aux * omega / diagonal[c];
                z_r_new_local += zirconium[c] * residual[c];
            }
            z_r_new += z_r_new_local;
        }
        const double beta = z_r_new / z_r;                    /* :1309-1318 */
        z_r = z_r_new;
        #pragma omp parallel for
        for (int c = 0; c < N; c++) {
            if (diagonal[c] == 0.0) continue;
            direction[c] = zirconium[c] + beta * direction[c];
        }
        K++;
    }
    free(direction); free(zirconium); free(auxiliary); free(mittlerer);
    return K;
}

/* Shared by both Eisenstat variants: work vectors start as NaN, as in the reference
 * (std::fill_n(..., notanumber)), so rows the sweeps skip stay NaN. */
static double* nan_vector(int N)
{
    double* v = (double*)malloc((size_t)(N > 0 ? N : 1) * sizeof(double));
    if (v) for (int i = 0; i < N; i++) v[i] = NAN;
    return v;
}

/* solver/sparsesolver.cpp:726-995, SSOR-PCG with Eisenstat's trick (index order); returns K.
 * The iteration works on the L-solved residual: `residual` holds it on return. */
int oracle_cg_ssor_eisenstat(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                             double* residual, double precision, int print_modulo,
                             const double* diagonal, double omega)
{
    (void)print_modulo;
    double tolerance = 0.0;                                   /* :750-753 */
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = precision * sqrt(tolerance);
    tolerance = dmax(tolerance, ORACLE_DESIRED_PRECISION);

    double* direction = nan_vector(N);                        /* :766-773 */
    double* zirconium = nan_vector(N);
    double* technical = nan_vector(N);
    double* auxiliary = nan_vector(N);
    if (!direction || !zirconium || !technical || !auxiliary) {
        free(direction); free(zirconium); free(technical); free(auxiliary); return -1;
    }
    double z_r = NAN;
    int K = 0;
    while (K < N) {
        if (K == 0) {                                         /* :786-842 */
            #pragma omp parallel for
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                double aux = b[c];
                for (int d = A[c]; d < A[c + 1]; d++)
                    if (diagonal[C[d]] != 0.0) aux -= V[d] * x[C[d]];
                auxiliary[c] = aux;
            }
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                double aux = auxiliary[c];
                for (int d = A[c]; d < A[c + 1]; d++)
                    if (C[d] < c && diagonal[C[d]] != 0.0) aux -= V[d] * residual[C[d]];
                residual[c] = aux * omega / diagonal[c];
            }
            z_r = 0.0;
            #pragma omp parallel for reduction(+:z_r)
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                zirconium[c] = residual[c] * diagonal[c] * (2.0 - omega) / omega;
                direction[c] = zirconium[c];
                z_r += zirconium[c] * residual[c];
            }
        }
        if (fabs(z_r) < tolerance * tolerance) break;        /* :859-862 */

        double d_Ad = 0.0;                                    /* :870-914 */
        for (int c = N - 1; c >= 0; c--) {
            if (diagonal[c] == 0.0) continue;
            double aux = direction[c];
            for (int d = A[c]; d < A[c + 1]; d++)
                if (C[d] > c && diagonal[C[d]] != 0.0) aux -= V[d] * technical[C[d]];
            technical[c] = aux * omega / diagonal[c];
        }
        for (int c = 0; c < N; c++) {
            if (diagonal[c] == 0.0) continue;
            double aux = direction[c] - (2.0 / omega - 1.0) * diagonal[c] * technical[c];
            for (int d = A[c]; d < A[c + 1]; d++)
                if (C[d] < c && diagonal[C[d]] != 0.0) aux -= V[d] * auxiliary[C[d]];
            auxiliary[c] = aux * omega / diagonal[c];
        }
        #pragma omp parallel for reduction(+:d_Ad)
        for (int c = 0; c < N; c++) {
            if (diagonal[c] == 0.0) continue;
            auxiliary[c] += technical[c];
            d_Ad += auxiliary[c] * direction[c];
        }
        int numerator_bad = !isfinite(z_r) || z_r < 0.0;      /* :918-933 */
        int denominator_bad = !isfinite(d_Ad) || d_Ad < 0.0;
        int denominator_small = sqrt(fabs(d_Ad)) < ORACLE_MACHINE_EPSILON;
        if (numerator_bad || denominator_bad) break;
        if (denominator_small) break;

        const double alpha = z_r / d_Ad;                      /* :936-975 */
        double z_r_new = 0.0;
        #pragma omp parallel for reduction(+:z_r_new)
        for (int c = 0; c < N; c++) {
            if (diagonal[c] == 0.0) continue;
            x[c] += alpha * technical[c];
            residual[c] -= alpha * auxiliary[c];
            zirconium[c] = residual[c] * (diagonal[c] * (2.0 - omega) / omega);
            z_r_new += zirconium[c] * residual[c];
        }
        const double beta = z_r_new / z_r;
        z_r = z_r_new;
        #pragma omp parallel for
        for (int c = 0; c < N; c++) {
            if (diagonal[c] == 0.0) continue;
            direction[c] = zirconium[c] + beta * direction[c];
        }
        K++;
    }
    free(direction); free(zirconium); free(technical); free(auxiliary);
    return K;
}

/* solver/sparsesolver.cpp:1338-1645, multicolor SSOR-PCG with Eisenstat's trick; returns K.
 * As in the reference, the column guard diagonal[col] != 0 applies in the restart only. */
int oracle_cg_eisenstat_rainbow(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                                double* residual, double precision, int print_modulo,
                                const double* diagonal, double omega,
                                int num_colors, const int* F, const int* B, const int* R)
{
    (void)print_modulo;
    double tolerance = 0.0;                                   /* :1367-1370 */
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = precision * sqrt(tolerance);
    tolerance = dmax(tolerance, ORACLE_DESIRED_PRECISION);

    double* direction = nan_vector(N);                        /* :1383-1394 */
    double* zirconium = nan_vector(N);
    double* technical = nan_vector(N);
    double* auxiliary = nan_vector(N);
    if (!direction || !zirconium || !technical || !auxiliary) {
        free(direction); free(zirconium); free(technical); free(auxiliary); return -1;
    }
    double z_r = NAN;
    int K = 0;
    while (K < N) {
        if (K == 0) {                                         /* :1409-1478 */
            #pragma omp parallel for
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                double aux = b[c];
                for (int d = A[c]; d < A[c + 1]; d++)
                    if (diagonal[C[d]] != 0.0) aux -= V[d] * x[C[d]];
                auxiliary[c] = aux;
            }
            for (int color = 0; color < num_colors; color++) {
                #pragma omp parallel for
                for (int i = B[color]; i < B[color + 1]; i++) {
                    const int c = R[i];
                    if (diagonal[c] == 0.0) continue;
                    double aux = auxiliary[c];
                    for (int d = A[c]; d < A[c + 1]; d++)
                        if (F[C[d]] < F[c] && diagonal[C[d]] != 0.0) aux -= V[d] * residual[C[d]];
                    residual[c] = aux * omega / diagonal[c];
                }
            }
            z_r = 0.0;
            #pragma omp parallel for reduction(+:z_r)
            for (int c = 0; c < N; c++) {
                if (diagonal[c] == 0.0) continue;
                zirconium[c] = residual[c] * diagonal[c] * (2.0 - omega) / omega;
                direction[c] = zirconium[c];
                z_r += zirconium[c] * residual[c];
            }
        }
        if (fabs(z_r) < tolerance * tolerance) break;        /* :1495-1498 */

        double d_Ad = 0.0;                                    /* :1506-1574 */
        for (int color = num_colors - 1; color >= 0; color--) {
            #pragma omp parallel for
            for (int i = B[color]; i < B[color + 1]; i++) {
                const int c = R[i];
                if (diagonal[c] == 0.0) continue;
                double aux = direction[c];
                for (int d = A[c]; d < A[c + 1]; d++)
                    if (F[C[d]] > F[c]) aux -= V[d] * technical[C[d]];
                technical[c] = aux * omega / diagonal[c];
            }
        }
        for (int color = 0; color < num_colors; color++) {
            #pragma omp parallel for
            for (int i = B[color]; i < B[color + 1]; i++) {
                const int c = R[i];
                if (diagonal[c] == 0.0) continue;
                double aux = direction[c] - (2.0 / omega - 1.0) * diagonal[c] * technical[c];
                for (int d = A[c]; d < A[c + 1]; d++)
                    if (F[C[d]] < F[c]) aux -= V[d] * auxiliary[C[d]];
                auxiliary[c] = aux * omega / diagonal[c];
            }
        }
        #pragma omp parallel for reduction(+:d_Ad)
        for (int c = 0; c < N; c++) {
            if (diagonal[c] == 0.0) continue;
            auxiliary[c] += technical[c];
            d_Ad += auxiliary[c] * direction[c];
        }
        int numerator_bad = !isfinite(z_r) || z_r < 0.0;      /* :1578-1593 */
        int denominator_bad = !isfinite(d_Ad) || d_Ad < 0.0;
        int denominator_small = sqrt(fabs(d_Ad)) < ORACLE_MACHINE_EPSILON;
        if (numerator_bad || denominator_bad) break;
        if (denominator_small) break;

        const double alpha = z_r / d_Ad;                      /* :1596-1629 */
        double z_r_new = 0.0;
        #pragma omp parallel for reduction(+:z_r_new)
        for (int c = 0; c < N; c++) {
            if (diagonal[c] == 0.0) continue;
            x[c] += alpha * technical[c];
            residual[c] -= alpha * auxiliary[c];
            zirconium[c] = residual[c] * (diagonal[c] * (2.0 - omega) / omega);
            z_r_new += zirconium[c] * residual[c];
        }
        const double beta = z_r_new / z_r;
        z_r = z_r_new;
        #pragma omp parallel for
        for (int c = 0; c < N; c++) {
            if (diagonal[c] == 0.0) continue;
            direction[c] = zirconium[c] + beta * direction[c];
        }
        K++;
    }
    free(direction); free(zirconium); free(technical); free(auxiliary);
    return K;
}

/* ---------------------------------------------------------------------------
 * CSR algebra (the step before the solver path)
 * ------------------------------------------------------------------------- */

/* sparse/matcsr.cpp:585-688 (sort_and_compress_csrdata_reduced), in place: per row, an
 * exchange sort by column that merges equal columns into the first (the later one set
 * to 0), a bubble pass that moves zeros to the end, the row keeps its entries before the
 * first zero; then the rows are compacted and A rebuilt. Returns the new entry count. */
int oracle_csr_compress(int rows, int* A, int* C, double* V)
{
    int* nnz = (int*)malloc((size_t)(rows > 0 ? rows : 1) * sizeof(int));
    if (!nnz) return -1;
    #pragma omp parallel for
    for (int r = 0; r < rows; r++) {
        for (int i = A[r]; i < A[r + 1]; i++)
            for (int j = i + 1; j < A[r + 1]; j++) {
                if (C[i] == C[j]) { V[i] += V[j]; V[j] = 0.0; continue; }
                if (C[i] > C[j]) {
                    const int tc = C[i]; C[i] = C[j]; C[j] = tc;
                    const double tv = V[i]; V[i] = V[j]; V[j] = tv;
                }
            }
        for (int i = A[r]; i < A[r + 1]; i++)
            for (int j = A[r] + 1; j < A[r + 1]; j++)
                if (V[j - 1] == 0.0 && V[j] != 0.0) {
                    const int tc = C[j - 1]; C[j - 1] = C[j]; C[j] = tc;
                    const double tv = V[j - 1]; V[j - 1] = V[j]; V[j] = tv;
                }
        int first_zero = A[r];
        while (first_zero < A[r + 1] && V[first_zero] != 0.0) first_zero++;
        nnz[r] = first_zero - A[r];
    }
    int target = 0;
    for (int r = 0; r < rows; r++)
        for (int i = A[r]; i < A[r] + nnz[r]; i++) { C[target] = C[i]; V[target] = V[i]; target++; }
    for (int r = 0; r < rows; r++) A[r + 1] = nnz[r];
    A[0] = 0;
    for (int r = 1; r <= rows; r++) A[r] += A[r - 1];
    free(nnz);
    return A[rows];
}

/* sparse/matcsr.cpp:707-765, MatrixCSRAddition: s1 * mat1 + s2 * mat2 (same shape). The
 * outputs hold A1[rows] + A2[rows] entries before compression; returns the final count. */
int oracle_csr_add(int rows, const int* A1, const int* C1, const double* V1, const int* A2, const int* C2,
                   const double* V2, double s1, double s2, int* A, int* C, double* V)
{
    A[0] = 0;
    for (int r = 1; r <= rows; r++) A[r] = A[r - 1] + (A1[r] - A1[r - 1]) + (A2[r] - A2[r - 1]);
    for (int r = 0; r < rows; r++) {
        int i = 0;
        for (int c1 = A1[r]; c1 < A1[r + 1]; c1++) C[A[r] + (i++)] = C1[c1];
        for (int c2 = A2[r]; c2 < A2[r + 1]; c2++) C[A[r] + (i++)] = C2[c2];
    }
    for (int r = 0; r < rows; r++) {
        int i = 0;
        for (int v1 = A1[r]; v1 < A1[r + 1]; v1++) V[A[r] + (i++)] = s1 * V1[v1];
        for (int v2 = A2[r]; v2 < A2[r + 1]; v2++) V[A[r] + (i++)] = s2 * V2[v2];
    }
    return oracle_csr_compress(rows, A, C, V);
}

/* sparse/matcsr.cpp:767-796: entries of mat1 * mat2 before compression (the capacity the
 * outputs of oracle_csr_multiply need). */
long long oracle_csr_multiply_size(int rows, const int* A1, const int* C1, const int* A2)
{
    long long total = 0;
    for (int r = 0; r < rows; r++)
        for (int c1 = A1[r]; c1 < A1[r + 1]; c1++) total += A2[C1[c1] + 1] - A2[C1[c1]];
    return total;
}

/* sparse/matcsr.cpp:767-849, MatrixCSRMultiplication: all products in row order, then
 * the compression above. Returns the final entry count. */
int oracle_csr_multiply(int rows, const int* A1, const int* C1, const double* V1, const int* A2, const int* C2,
                        const double* V2, int* A, int* C, double* V)
{
    A[0] = 0;
    for (int r = 0; r < rows; r++) {
        int cnt = 0;
        for (int c1 = A1[r]; c1 < A1[r + 1]; c1++) cnt += A2[C1[c1] + 1] - A2[C1[c1]];
        A[r + 1] = A[r] + cnt;
    }
    #pragma omp parallel for
    for (int r = 0; r < rows; r++) {
        int cur = A[r];
        for (int c1 = A1[r]; c1 < A1[r + 1]; c1++)
            for (int c2 = A2[C1[c1]]; c2 < A2[C1[c1] + 1]; c2++) {
                C[cur] = C2[c2];
                V[cur] = V1[c1] * V2[c2];
                cur++;
            }
    }
    return oracle_csr_compress(rows, A, C, V);
}

/* sparse/matcsr.cpp:291-350, MatrixCSR::getTranspose: entries bucketed by column, each
 * column filled from its end in row order, then the compression above. Returns the count. */
int oracle_csr_transpose(int rows, int cols, const int* A, const int* C, const double* V, int* B, int* D, double* W)
{
    const int nnz = A[rows];
    int* Z = (int*)calloc((size_t)(cols > 0 ? cols : 1), sizeof(int));
    if (!Z) return -1;
    for (int i = 0; i < nnz; i++) Z[C[i]]++;
    B[0] = 0;
    for (int c = 1; c <= cols; c++) B[c] = B[c - 1] + Z[c - 1];
    for (int r = 0; r < rows; r++)
        for (int i = A[r]; i < A[r + 1]; i++) {
            const int c = C[i];
            const int index = --Z[c];
            D[B[c] + index] = r;
            W[B[c] + index] = V[i];
        }
    free(Z);
    return oracle_csr_compress(cols, B, D, W);
}

/* sparse/matcsr.cpp:43-89 with sparse/sparsematrix.cpp:405-458: MatrixCSR(SparseMatrix).
 * Entries with value 0 are dropped, the rest sorted by (row, column) and equal positions
 * summed in sorted order (the reference's std::sort leaves equal keys in an unspecified
 * order; this sort is stable, so equal keys are summed in input order), then laid out as
 * CSR. Returns the entry count (A, C, V need `count` entries of room). */
typedef struct { int r, c; double v; long long i; } OracleEntry;
static int entry_cmp(const void* pa, const void* pb)
{
    const OracleEntry* a = (const OracleEntry*)pa; const OracleEntry* b = (const OracleEntry*)pb;
    if (a->r != b->r) return a->r < b->r ? -1 : 1;
    if (a->c != b->c) return a->c < b->c ? -1 : 1;
    return a->i < b->i ? -1 : (a->i > b->i);
}
int oracle_coo_to_csr(int rows, long long count, const int* r, const int* c, const double* v, int* A, int* C,
                      double* V)
{
    OracleEntry* e = (OracleEntry*)malloc((size_t)(count > 0 ? count : 1) * sizeof(OracleEntry));
    if (!e) return -1;
    long long m = 0;
    for (long long i = 0; i < count; i++)
        if (v[i] != 0.0) { e[m].r = r[i]; e[m].c = c[i]; e[m].v = v[i]; e[m].i = i; m++; }
    qsort(e, (size_t)m, sizeof(OracleEntry), entry_cmp);
    long long dest = 0;
    for (long long src = 1; src < m; src++) {
        if (e[src].r == e[dest].r && e[src].c == e[dest].c) e[dest].v += e[src].v;
        else e[++dest] = e[src];
    }
    const long long n = m > 0 ? dest + 1 : 0;
    for (int k = 0; k <= rows; k++) A[k] = 0;
    for (long long i = 0; i < n; i++) { A[e[i].r + 1] += 1; C[i] = e[i].c; V[i] = e[i].v; }
    for (int k = 1; k <= rows; k++) A[k] += A[k - 1];
    free(e);
    return (int)n;
}

/* solver/sparsesolver.cpp:1687-1915, ConjugateResidualSolverCSR (and the arithmetically
 * identical _textbook variant, :1918-2156); returns K. The loops carry the reference's
 * OpenMP clauses (:1751, :1768, :1836, :1859): identical bits at one thread. */
int oracle_cr(int N, double* x, const double* b, const int* A, const int* C, const double* V,
              double* res, double precision, int print_modulo)
{
    (void)print_modulo;
    double tolerance = 0.0;                                   /* :1709-1712 */
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = precision * sqrt(tolerance);
    tolerance = dmax(tolerance, ORACLE_DESIRED_PRECISION);
    double* dir = nan_vector(N); double* Adir = nan_vector(N); double* Ares = nan_vector(N);
    double* vil = nan_vector(N);
    if (!dir || !Adir || !Ares || !vil) { free(dir); free(Adir); free(Ares); free(vil); return -1; }
    double Ad_r = NAN, Ad_Ad = NAN;
    int K = 0;
    while (K < N) {
        if (K == 0) {                                         /* :1749-1790 */
            #pragma omp parallel for
            for (int c = 0; c < N; c++) {
                res[c] = b[c];
                for (int d = A[c]; d < A[c + 1]; d++) res[c] -= V[d] * x[C[d]];
                dir[c] = res[c];
            }
            Ad_r = 0.0; Ad_Ad = 0.0;
            #pragma omp parallel for reduction(+:Ad_r,Ad_Ad)
            for (int c = 0; c < N; c++) {
                Adir[c] = 0.0;
                for (int e = A[c]; e < A[c + 1]; e++) Adir[c] += V[e] * dir[C[e]];
                Ares[c] = Adir[c];
                Ad_r += Adir[c] * res[c];
                Ad_Ad += Adir[c] * Adir[c];
            }
        }
        if (!isfinite(Ad_r) || Ad_r < 0.0) break;             /* :1804-1815 */
        if (fabs(Ad_r) < tolerance * tolerance) break;
        if (!isfinite(Ad_Ad) || Ad_Ad < 0.0) break;           /* :1819-1833 */
        if (sqrt(fabs(Ad_Ad)) < ORACLE_MACHINE_EPSILON) break;
        const double alpha = Ad_r / Ad_Ad;                    /* :1840-1865 */
        double new_Ar_r = 0.0;
        #pragma omp parallel for reduction(+:new_Ar_r)
        for (int c = 0; c < N; c++) {
            vil[c] = 0.0;
            for (int d = A[c]; d < A[c + 1]; d++) vil[c] += V[d] * Adir[C[d]];
            x[c] = x[c] + alpha * dir[c];
            res[c] = res[c] - alpha * Adir[c];
            Ares[c] = Ares[c] - alpha * vil[c];
            new_Ar_r += Ares[c] * res[c];
        }
        const double beta = new_Ar_r / Ad_r;                  /* :1867-1882 */
        Ad_Ad = 0.0;
        #pragma omp parallel for reduction(+:Ad_Ad)
        for (int c = 0; c < N; c++) {
            dir[c] = res[c] + beta * dir[c];
            Adir[c] = Ares[c] + beta * Adir[c];
            Ad_Ad += Adir[c] * Adir[c];
        }
        Ad_r = new_Ar_r;
        K++;
    }
    free(dir); free(Adir); free(Ares); free(vil);
    return K;
}

/* solver/sparsesolver.cpp:2159-2425, MINRESCSR; returns K (res = b - A x at the end). The
 * loops carry the reference's OpenMP clauses (:2238, :2259, :2289, :2305, :2320, :2336). */
int oracle_minres(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                  double* res, double precision, int print_modulo)
{
    (void)print_modulo;
    double tolerance = 0.0;                                   /* :2181-2184 */
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = precision * sqrt(tolerance);
    tolerance = dmax(tolerance, ORACLE_DESIRED_PRECISION);
    double* v0 = nan_vector(N); double* v1 = nan_vector(N); double* w0 = nan_vector(N); double* w1 = nan_vector(N);
    double* vn = nan_vector(N); double* wn = nan_vector(N); double* p = nan_vector(N);
    if (!v0 || !v1 || !w0 || !w1 || !vn || !wn || !p) {
        free(v0); free(v1); free(w0); free(w1); free(vn); free(wn); free(p); return -1;
    }
    double gamma = NAN, eta = NAN, s0 = NAN, s1 = NAN, c0 = NAN, c1 = NAN;
    int K = 0;
    while (K < N) {
        if (K == 0) {                                         /* :2233-2283 */
            double gamma_sq = 0.0;
            #pragma omp parallel for reduction(+:gamma_sq)
            for (int c = 0; c < N; c++) {
                v0[c] = 0.0; w0[c] = 0.0; v1[c] = b[c]; w1[c] = 0.0;
                for (int d = A[c]; d < A[c + 1]; d++) v1[c] -= V[d] * x[C[d]];
                gamma_sq += v1[c] * v1[c];
            }
            gamma = sqrt(gamma_sq);
            #pragma omp parallel for
            for (int c = 0; c < N; c++) v1[c] /= gamma;
            s0 = s1 = 0.0;
            c0 = c1 = 1.0;
            eta = gamma;
        }
        if (fabs(eta) < tolerance) break;                     /* :2290-2293 */
        double delta = 0.0;                                   /* :2297-2313 */
        #pragma omp parallel for reduction(+:delta)
        for (int c = 0; c < N; c++) {
            p[c] = 0.0;
            for (int d = A[c]; d < A[c + 1]; d++) p[c] += V[d] * v1[C[d]];
            delta += p[c] * v1[c];
        }
        double gamma_n_sq = 0.0;                              /* :2317-2330 */
        #pragma omp parallel for reduction(+:gamma_n_sq)
        for (int c = 0; c < N; c++) {
            vn[c] = p[c] - delta * v1[c] - gamma * v0[c];
            gamma_n_sq += vn[c] * vn[c];
        }
        const double gamma_n = sqrt(gamma_n_sq);
        #pragma omp parallel for
        for (int c = 0; c < N; c++) vn[c] /= gamma_n;
        const double alpha_0 = c1 * delta - c0 * s1 * gamma; /* :2338-2349 */
        const double alpha_1 = sqrt(alpha_0 * alpha_0 + gamma_n * gamma_n);
        const double alpha_2 = s1 * delta + c0 * c1 * gamma;
        const double alpha_3 = s0 * gamma;
        const double cn = alpha_0 / alpha_1;
        const double sn = gamma_n / alpha_1;
        #pragma omp parallel for
        for (int c = 0; c < N; c++) {                         /* :2353-2360 */
            wn[c] = (v1[c] - alpha_2 * w1[c] - alpha_3 * w0[c]) / alpha_1;
            x[c] = x[c] + cn * eta * wn[c];
        }
        eta = -sn * eta;                                      /* :2362-2378 */
        double* t;
        t = v0; v0 = v1; v1 = t;
        t = w0; w0 = w1; w1 = t;
        t = v1; v1 = vn; vn = t;
        t = w1; w1 = wn; wn = t;
        gamma = gamma_n;
        c0 = c1; s0 = s1; c1 = cn; s1 = sn;
        K++;
    }
    for (int c = 0; c < N; c++) {                             /* :2397-2403 */
        res[c] = b[c];
        for (int d = A[c]; d < A[c + 1]; d++) res[c] -= V[d] * x[C[d]];
    }
    free(v0); free(v1); free(w0); free(w1); free(vn); free(wn); free(p);
    return K;
}

/* solver/sparsesolver.cpp:2428-2590, ChebyshevIteration_DiagonalPreconditioner; returns K.
 * As in the reference, x receives x_next after the last rotation of the three iterates. */
int oracle_chebyshev(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                     double* residual, double precision, int print_modulo, const double* precon,
                     double lower, double upper)
{
    (void)print_modulo;
    double tolerance = 0.0;                                   /* :2452-2455 */
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = precision * sqrt(tolerance);
    tolerance = dmax(tolerance, ORACLE_DESIRED_PRECISION);
    double* z = (double*)malloc(sizeof(double) * (size_t)(N > 0 ? N : 1));
    double* x_prev = nan_vector(N); double* x_curr = nan_vector(N); double* x_next = nan_vector(N);
    if (!z || !x_prev || !x_curr || !x_next) { free(z); free(x_prev); free(x_curr); free(x_next); return -1; }
    for (int c = 0; c < N; c++) x_prev[c] = x_curr[c] = x_next[c] = x[c];
    const double alpha = 2. / (upper + lower);                /* :2486-2487 */
    const double mu = (upper + lower) / (upper - lower);
    double gamma_prev = NAN, gamma_curr = NAN, r_r = NAN;
    int K = 0;
    while (K < N) {
        if (K == 0) {                                         /* :2499-2531 */
            gamma_prev = 1.;
            gamma_curr = mu;
            r_r = 0.;
            for (int c = 0; c < N; c++) x_prev[c] = x[c];
            for (int c = 0; c < N; c++) {
                residual[c] = b[c];
                for (int d = A[c]; d < A[c + 1]; d++) residual[c] -= V[d] * x_prev[C[d]];
                z[c] = precon[c] * residual[c];
                x_curr[c] = x_prev[c] + alpha * z[c];
                r_r += residual[c] * residual[c];
            }
        }
        if (sqrt(r_r) < tolerance) break;                     /* :2535-2538 */
        const double gamma_next = 2. * mu * gamma_curr - gamma_prev;   /* :2542-2563 */
        const double omega = 2. * mu * gamma_curr / gamma_next;
        r_r = 0.;
        for (int c = 0; c < N; c++) {
            residual[c] = b[c];
            for (int d = A[c]; d < A[c + 1]; d++) residual[c] -= V[d] * x_curr[C[d]];
            z[c] = precon[c] * residual[c];
            x_next[c] = x_prev[c] + omega * (alpha * z[c] + x_curr[c] - x_prev[c]);
            r_r += residual[c] * residual[c];
        }
        gamma_prev = gamma_curr;
        gamma_curr = gamma_next;
        double* t;
        t = x_curr; x_curr = x_prev; x_prev = t;
        t = x_next; x_next = x_curr; x_curr = t;
        K++;
    }
    for (int c = 0; c < N; c++) x[c] = x_next[c];              /* :2578-2582 */
    free(z); free(x_prev); free(x_curr); free(x_next);
    return K;
}

/* solver/systemsparsesolver.cpp:52-1120, the Hodge conjugate residual solvers: conjugate
 * residuals on M = B A^-1 Bt + C (N x N; A is L x L, B N x L, Bt L x N), A^-1 applied by an
 * inner CG to inner_precision: variant 0 diagonally preconditioned (precon = 1 / the
 * diagonal, :76-91; HodgeConjugateResidualSolverCSR_diagonal), 1 SSOR with omega = 1
 * (:500-516; _SSOR and HodgeConjugateResidualSolverCSR), 2 plain CG (_textbook). The inner
 * solve of each restart starts from zero, those of the iterations from the previous inner
 * solution (:253-277). Returns K. The loops carry the reference's OpenMP clauses (:126,
 * :162, :186, :206, :230, :298, :322, :357): identical bits at one thread. */
int oracle_hodge_cr(int variant, int N, int L, double* x, const double* b,
                    const int* Ar, const int* Ac, const double* Av, const int* Br, const int* Bc, const double* Bv,
                    const int* Btr, const int* Btc, const double* Btv, const int* Cr, const int* Cc, const double* Cv,
                    double* res, double precision, double inner_precision)
{
    const double sign_A = 1.;                                 /* systemsparsesolver.hpp:8 */
    double tolerance = 0.0;
    for (int i = 0; i < N; i++) tolerance += b[i] * b[i];
    tolerance = precision * sqrt(tolerance);
    tolerance = dmax(tolerance, ORACLE_DESIRED_PRECISION);
    double* dir = (double*)malloc(sizeof(double) * (size_t)N);
    double* Mdir = (double*)malloc(sizeof(double) * (size_t)N);
    double* Mres = (double*)malloc(sizeof(double) * (size_t)N);
    double* vil = (double*)malloc(sizeof(double) * (size_t)N);
    double* aux1 = (double*)malloc(sizeof(double) * (size_t)L);
    double* aux2 = (double*)malloc(sizeof(double) * (size_t)L);
    double* auxR = (double*)malloc(sizeof(double) * (size_t)L);
    double* diag = (double*)malloc(sizeof(double) * (size_t)L);
    if (!dir || !Mdir || !Mres || !vil || !aux1 || !aux2 || !auxR || !diag) {
        free(dir); free(Mdir); free(Mres); free(vil); free(aux1); free(aux2); free(auxR); free(diag); return -1;
    }
    #pragma omp parallel for
    for (int c = 0; c < L; c++) {                             /* :76-91 / :500-516 */
        diag[c] = 0.;
        for (int d = Ar[c]; d < Ar[c + 1]; d++) if (Ac[d] == c) diag[c] += Av[d];
        if (variant == 0) diag[c] = 1. / diag[c];
    }
#define HODGE_INNER(xx, bb)                                                                          \
    do {                                                                                            \
        if (variant == 0) oracle_cg_diag(L, xx, bb, Ar, Ac, Av, auxR, inner_precision, -3, diag);   \
        else if (variant == 1) oracle_cg_ssor(L, xx, bb, Ar, Ac, Av, auxR, inner_precision, -3, diag, 1.); \
        else oracle_cg(L, xx, bb, Ar, Ac, Av, auxR, inner_precision, -3);                           \
    } while (0)
    double Md_r = NAN, Md_Md = NAN;
    int K = 0;
    while (K < N) {
        if (K == 0) {                                         /* :107-200 */
            #pragma omp parallel for
            for (int c = 0; c < L; c++) {
                aux1[c] = 0.;
                for (int d = Btr[c]; d < Btr[c + 1]; d++) aux1[c] += Btv[d] * x[Btc[d]];
            }
            for (int c = 0; c < L; c++) aux2[c] = 0.;
            HODGE_INNER(aux2, aux1);
            #pragma omp parallel for
            for (int c = 0; c < N; c++) {
                res[c] = b[c];
                for (int d = Br[c]; d < Br[c + 1]; d++) res[c] -= sign_A * Bv[d] * aux2[Bc[d]];
                for (int d = Cr[c]; d < Cr[c + 1]; d++) res[c] -= Cv[d] * x[Cc[d]];
                dir[c] = res[c];
            }
            Md_r = 0.; Md_Md = 0.;
            #pragma omp parallel for
            for (int c = 0; c < L; c++) {
                aux1[c] = 0;
                for (int d = Btr[c]; d < Btr[c + 1]; d++) aux1[c] += Btv[d] * dir[Btc[d]];
            }
            for (int c = 0; c < L; c++) aux2[c] = 0.;
            HODGE_INNER(aux2, aux1);
            #pragma omp parallel for reduction(+:Md_r,Md_Md)
            for (int c = 0; c < N; c++) {
                Mdir[c] = 0.;
                for (int d = Br[c]; d < Br[c + 1]; d++) Mdir[c] += sign_A * Bv[d] * aux2[Bc[d]];
                for (int d = Cr[c]; d < Cr[c + 1]; d++) Mdir[c] += Cv[d] * dir[Cc[d]];
                Mres[c] = Mdir[c];
                Md_r += Mdir[c] * res[c];
                Md_Md += Mdir[c] * Mdir[c];
            }
        }
        if (!isfinite(Md_r) || Md_r < 0.) break;             /* :212-222 */
        if (fabs(Md_r) < tolerance * tolerance) break;
        if (!isfinite(Md_Md) || Md_Md < 0.) break;           /* :224-238 */
        if (sqrt(fabs(Md_Md)) < ORACLE_MACHINE_EPSILON) break;
        const double alpha = Md_r / Md_Md;                    /* :242-300 */
        double new_Mr_r = 0.;
        #pragma omp parallel for
        for (int c = 0; c < L; c++) {
            aux1[c] = 0.;
            for (int d = Btr[c]; d < Btr[c + 1]; d++) aux1[c] += Btv[d] * Mdir[Btc[d]];
        }
        HODGE_INNER(aux2, aux1);
        #pragma omp parallel for reduction(+:new_Mr_r)
        for (int c = 0; c < N; c++) {
            vil[c] = 0.;
            for (int d = Br[c]; d < Br[c + 1]; d++) vil[c] += sign_A * Bv[d] * aux2[Bc[d]];
            for (int d = Cr[c]; d < Cr[c + 1]; d++) vil[c] += Cv[d] * Mdir[Cc[d]];
            x[c] = x[c] + alpha * dir[c];
            res[c] = res[c] - alpha * Mdir[c];
            Mres[c] = Mres[c] - alpha * vil[c];
            new_Mr_r += Mres[c] * res[c];
        }
        const double beta = new_Mr_r / Md_r;                  /* :302-318 */
        Md_Md = 0.;
        #pragma omp parallel for reduction(+:Md_Md)
        for (int c = 0; c < N; c++) {
            dir[c] = res[c] + beta * dir[c];
            Mdir[c] = Mres[c] + beta * Mdir[c];
            Md_Md += Mdir[c] * Mdir[c];
        }
        Md_r = new_Mr_r;
        K++;
    }
#undef HODGE_INNER
    free(dir); free(Mdir); free(Mres); free(vil); free(aux1); free(aux2); free(auxR); free(diag);
    return K;
}

/* solver/systemsparsesolver.cpp:1122-1575, HodgeHerzogSoodhalterMethod: preconditioned
 * MINRES on [[-A, Bt], [B, C]] [x_A; x_C] = [b_A; b_C] with the block preconditioner
 * diag(PA, PC) applied by inner CG solves (each block skipped when its matrix is absent:
 * PAr == NULL / PCr == NULL). Returns the iteration count. */
static double odot(int n, const double* a, const double* b)
{
    double s = 0.;
    for (int i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

int oracle_hodge_hs(int dA, int dC, double* x_A, double* x_C, const double* b_A, const double* b_C,
                    const int* Ar, const int* Ac, const double* Av, const int* Br, const int* Bc, const double* Bv,
                    const int* Btr, const int* Btc, const double* Btv, const int* Cr, const int* Cc, const double* Cv,
                    double precision, const int* PAr, const int* PAc, const double* PAv,
                    const int* PCr, const int* PCc, const double* PCv, double inner_precision)
{
    const double sign_A = 1.;
    double tolerance = 0.;                                    /* :1167-1171 */
    for (int i = 0; i < dA; i++) tolerance += b_A[i] * b_A[i];
    for (int i = 0; i < dC; i++) tolerance += b_C[i] * b_C[i];
    tolerance = precision * sqrt(tolerance);
    tolerance = dmax(tolerance, ORACLE_DESIRED_PRECISION);
    double *v0_A = nan_vector(dA), *v1_A = nan_vector(dA), *w0_A = nan_vector(dA), *w1_A = nan_vector(dA);
    double *z_A = nan_vector(dA), *vn_A = nan_vector(dA), *wn_A = nan_vector(dA), *zn_A = nan_vector(dA);
    double *m_A = nan_vector(dA), *p_A = nan_vector(dA);
    double *v0_C = nan_vector(dC), *v1_C = nan_vector(dC), *w0_C = nan_vector(dC), *w1_C = nan_vector(dC);
    double *z_C = nan_vector(dC), *vn_C = nan_vector(dC), *wn_C = nan_vector(dC), *zn_C = nan_vector(dC);
    double *m_C = nan_vector(dC), *p_C = nan_vector(dC);
    double* all[] = {v0_A, v1_A, w0_A, w1_A, z_A, vn_A, wn_A, zn_A, m_A, p_A,
                     v0_C, v1_C, w0_C, w1_C, z_C, vn_C, wn_C, zn_C, m_C, p_C};
    for (int k = 0; k < 20; k++) if (!all[k]) { for (int j = 0; j < 20; j++) free(all[j]); return -1; }
    double mu_A = NAN, mu_C = NAN, gamma = NAN, eta = NAN, eta_A = NAN, eta_C = NAN;
    double s0 = NAN, s1 = NAN, c0 = NAN, c1 = NAN;
    const int max_iteration_count = dA + dC;
    int count = 0;
    const int pa = PAr && PAc && PAv, pc = PCr && PCc && PCv;
    (void)mu_A; (void)mu_C; (void)eta_A; (void)eta_C;
    while (count < max_iteration_count) {
        if (count == 0) {                                     /* :1240-1330 */
            for (int a = 0; a < dA; a++) v0_A[a] = w0_A[a] = w1_A[a] = 0.;
            for (int c = 0; c < dC; c++) v0_C[c] = w0_C[c] = w1_C[c] = 0.;
            for (int r = 0; r < dA; r++) {
                v1_A[r] = b_A[r];
                for (int d = Ar[r]; d < Ar[r + 1]; d++) v1_A[r] += sign_A * Av[d] * x_A[Ac[d]];
                for (int d = Btr[r]; d < Btr[r + 1]; d++) v1_A[r] -= Btv[d] * x_C[Btc[d]];
            }
            for (int r = 0; r < dC; r++) {
                v1_C[r] = b_C[r];
                for (int d = Br[r]; d < Br[r + 1]; d++) v1_C[r] -= Bv[d] * x_A[Bc[d]];
                for (int d = Cr[r]; d < Cr[r + 1]; d++) v1_C[r] -= Cv[d] * x_C[Cc[d]];
            }
            for (int r = 0; r < dA; r++) z_A[r] = v1_A[r];
            for (int r = 0; r < dC; r++) z_C[r] = v1_C[r];
            if (pa) oracle_cg(dA, z_A, v1_A, PAr, PAc, PAv, wn_A, inner_precision, -3);
            if (pc) oracle_cg(dC, z_C, v1_C, PCr, PCc, PCv, wn_C, inner_precision, -3);
            const double v1_z_A = odot(dA, v1_A, z_A);
            const double v1_z_C = odot(dC, v1_C, z_C);
            gamma = sqrt(v1_z_A + v1_z_C);
            for (int a = 0; a < dA; a++) { v1_A[a] /= gamma; z_A[a] /= gamma; m_A[a] = v1_A[a]; }
            for (int c = 0; c < dC; c++) { v1_C[c] /= gamma; z_C[c] /= gamma; m_C[c] = v1_C[c]; }
            const double psi_A = v1_z_A / (gamma * gamma);
            const double psi_C = v1_z_C / (gamma * gamma);
            mu_A = psi_A; mu_C = psi_C;
            eta = gamma;
            eta_A = gamma * sqrt(psi_A); eta_C = gamma * sqrt(psi_C);
            s0 = s1 = 0.;
            c0 = c1 = 1.;
        }
        if (fabs(eta) < tolerance) break;                     /* :1336-1339 */
        double z_p_A = 0., z_p_C = 0.;                        /* :1345-1371 */
        for (int r = 0; r < dA; r++) {
            p_A[r] = 0.;
            for (int d = Ar[r]; d < Ar[r + 1]; d++) p_A[r] -= sign_A * Av[d] * z_A[Ac[d]];
            for (int d = Btr[r]; d < Btr[r + 1]; d++) p_A[r] += Btv[d] * z_C[Btc[d]];
            z_p_A += p_A[r] * z_A[r];
        }
        for (int r = 0; r < dC; r++) {
            p_C[r] = 0.;
            for (int d = Br[r]; d < Br[r + 1]; d++) p_C[r] += Bv[d] * z_A[Bc[d]];
            for (int d = Cr[r]; d < Cr[r + 1]; d++) p_C[r] += Cv[d] * z_C[Cc[d]];
            z_p_C += p_C[r] * z_C[r];
        }
        const double delta = z_p_A + z_p_C;
        for (int a = 0; a < dA; a++) vn_A[a] = p_A[a] - delta * v1_A[a] - gamma * v0_A[a];
        for (int c = 0; c < dC; c++) vn_C[c] = p_C[c] - delta * v1_C[c] - gamma * v0_C[c];
        double zn_vn_A = 0., zn_vn_C = 0.;
        for (int a = 0; a < dA; a++) { zn_A[a] = vn_A[a]; zn_vn_A += zn_A[a] * vn_A[a]; }
        for (int c = 0; c < dC; c++) { zn_C[c] = vn_C[c]; zn_vn_C += zn_C[c] * vn_C[c]; }
        if (pa) { oracle_cg(dA, zn_A, vn_A, PAr, PAc, PAv, wn_A, inner_precision, -3); zn_vn_A = odot(dA, zn_A, vn_A); }
        if (pc) { oracle_cg(dC, zn_C, vn_C, PCr, PCc, PCv, wn_C, inner_precision, -3); zn_vn_C = odot(dC, zn_C, vn_C); }
        const double gamma_n = sqrt(zn_vn_A + zn_vn_C);
        for (int a = 0; a < dA; a++) { vn_A[a] /= gamma_n; zn_A[a] /= gamma_n; }
        for (int c = 0; c < dC; c++) { vn_C[c] /= gamma_n; zn_C[c] /= gamma_n; }
        const double alpha_0 = c1 * delta - c0 * s1 * gamma;
        const double alpha_1 = sqrt(alpha_0 * alpha_0 + gamma_n * gamma_n);
        const double alpha_2 = s1 * delta + c0 * c1 * gamma;
        const double alpha_3 = s0 * gamma;
        const double cn = alpha_0 / alpha_1;
        const double sn = gamma_n / alpha_1;
        double theta_A = 0., theta_C = 0., psi_A = 0., psi_C = 0.;
        for (int a = 0; a < dA; a++) { theta_A += m_A[a] * zn_A[a]; psi_A += zn_A[a] * vn_A[a]; }
        for (int c = 0; c < dC; c++) { theta_C += m_C[c] * zn_C[c]; psi_C += zn_C[c] * vn_C[c]; }
        for (int a = 0; a < dA; a++) {
            m_A[a] = -sn * m_A[a] + cn * vn_A[a];
            wn_A[a] = (z_A[a] - alpha_3 * w0_A[a] - alpha_2 * w1_A[a]) / alpha_1;
            x_A[a] = x_A[a] + cn * eta * wn_A[a];
        }
        for (int c = 0; c < dC; c++) {
            m_C[c] = -sn * m_C[c] + cn * vn_C[c];
            wn_C[c] = (z_C[c] - alpha_3 * w0_C[c] - alpha_2 * w1_C[c]) / alpha_1;
            x_C[c] = x_C[c] + cn * eta * wn_C[c];
        }
        mu_A = sn * sn * mu_A - 2 * sn * cn * theta_A + cn * cn * psi_A;
        mu_C = sn * sn * mu_C - 2 * sn * cn * theta_C + cn * cn * psi_C;
        eta = -sn * eta;
        eta_A = eta * sqrt(psi_A); eta_C = eta * sqrt(psi_C);
        double* t;                                            /* :1494-1503 */
        t = v0_A; v0_A = v1_A; v1_A = t; t = v1_A; v1_A = vn_A; vn_A = t;
        t = v0_C; v0_C = v1_C; v1_C = t; t = v1_C; v1_C = vn_C; vn_C = t;
        t = w0_A; w0_A = w1_A; w1_A = t; t = w1_A; w1_A = wn_A; wn_A = t;
        t = w0_C; w0_C = w1_C; w1_C = t; t = w1_C; w1_C = wn_C; wn_C = t;
        t = z_A; z_A = zn_A; zn_A = t;
        t = z_C; z_C = zn_C; zn_C = t;
        gamma = gamma_n;
        c0 = c1; c1 = cn;
        s0 = s1; s1 = sn;
        count++;
    }
    double* fin[] = {v0_A, v1_A, w0_A, w1_A, z_A, vn_A, wn_A, zn_A, m_A, p_A,
                     v0_C, v1_C, w0_C, w1_C, z_C, vn_C, wn_C, zn_C, m_C, p_C};
    for (int j = 0; j < 20; j++) free(fin[j]);
    return count;
}

/* sparse/sparsematrix.cpp:609-722, SparseMatrixMultiplication(left, right), with
 * SparseMatrix::sortandcompressentries (:405-458) for the operands and the result.
 * Operands: zeros dropped, sorted (left by column then row, right by row then column),
 * equal positions summed in sorted order. Every product L(i,k) R(k,j) is emitted in the
 * order k, then i, then j; the result drops zero products, is sorted by row then column
 * and sums equal positions in sorted order. The reference's std::sort leaves the order of
 * equal positions unspecified; these sorts are stable (input order, then emission order:
 * k ascending). Entries are returned row-wise sorted. */
static long long compress_entries(long long count, const int* r, const int* c, const double* v, int colwise,
                                  OracleEntry* e)
{
    long long m = 0;
    for (long long i = 0; i < count; i++)
        if (v[i] != 0.0) {
            e[m].r = colwise ? c[i] : r[i]; e[m].c = colwise ? r[i] : c[i];
            e[m].v = v[i]; e[m].i = i; m++;
        }
    qsort(e, (size_t)m, sizeof(OracleEntry), entry_cmp);
    if (m == 0) return 0;
    long long dest = 0;
    for (long long src = 1; src < m; src++) {
        if (e[src].r == e[dest].r && e[src].c == e[dest].c) e[dest].v += e[src].v;
        else e[++dest] = e[src];
    }
    return dest + 1;
}

/* Upper bound on the products emitted (before any compression): for every k, the left
 * entries in column k times the right entries in row k. */
long long oracle_coo_multiply_size(int inner, long long ln, const int* lc, long long rn, const int* rr)
{
    long long* a = (long long*)calloc((size_t)(inner > 0 ? inner : 1), sizeof(long long));
    long long* b = (long long*)calloc((size_t)(inner > 0 ? inner : 1), sizeof(long long));
    long long total = 0;
    if (!a || !b) { free(a); free(b); return -1; }
    for (long long i = 0; i < ln; i++) a[lc[i]]++;
    for (long long i = 0; i < rn; i++) b[rr[i]]++;
    for (int k = 0; k < inner; k++) total += a[k] * b[k];
    free(a); free(b);
    return total;
}

long long oracle_coo_multiply(long long ln, const int* lr, const int* lc, const double* lv,
                              long long rn, const int* rr, const int* rc, const double* rv,
                              int* out_r, int* out_c, double* out_v)
{
    OracleEntry* le = (OracleEntry*)malloc((size_t)(ln > 0 ? ln : 1) * sizeof(OracleEntry));
    OracleEntry* re = (OracleEntry*)malloc((size_t)(rn > 0 ? rn : 1) * sizeof(OracleEntry));
    if (!le || !re) { free(le); free(re); return -1; }
    const long long lnum = compress_entries(ln, lr, lc, lv, 1, le);   /* (column k, row i) */
    const long long rnum = compress_entries(rn, rr, rc, rv, 0, re);   /* (row k, column j) */
    long long cap = 0;
    for (long long lb = 0, rb = 0; lb < lnum && rb < rnum;) {
        if (le[lb].r == re[rb].r) {
            const int k = le[lb].r;
            long long ln2 = lb, rn2 = rb;
            while (ln2 < lnum && le[ln2].r == k) ln2++;
            while (rn2 < rnum && re[rn2].r == k) rn2++;
            cap += (ln2 - lb) * (rn2 - rb);
            lb = ln2; rb = rn2;
        } else if (le[lb].r < re[rb].r) lb++; else rb++;
    }
    OracleEntry* pe = (OracleEntry*)malloc((size_t)(cap > 0 ? cap : 1) * sizeof(OracleEntry));
    if (!pe) { free(le); free(re); return -1; }
    long long m = 0;
    for (long long lb = 0, rb = 0; lb < lnum && rb < rnum;) {
        if (le[lb].r == re[rb].r) {
            const int k = le[lb].r;
            long long ln2 = lb, rn2 = rb;
            while (ln2 < lnum && le[ln2].r == k) ln2++;
            while (rn2 < rnum && re[rn2].r == k) rn2++;
            for (long long a = lb; a < ln2; a++)
                for (long long b = rb; b < rn2; b++) {
                    const double prod = le[a].v * re[b].v;
                    if (prod != 0.0) { pe[m].r = le[a].c; pe[m].c = re[b].c; pe[m].v = prod; pe[m].i = m; m++; }
                }
            lb = ln2; rb = rn2;
        } else if (le[lb].r < re[rb].r) lb++; else rb++;
    }
    qsort(pe, (size_t)m, sizeof(OracleEntry), entry_cmp);
    long long n = 0;
    if (m > 0) {
        long long dest = 0;
        for (long long src = 1; src < m; src++) {
            if (pe[src].r == pe[dest].r && pe[src].c == pe[dest].c) pe[dest].v += pe[src].v;
            else pe[++dest] = pe[src];
        }
        n = dest + 1;
    }
    for (long long i = 0; i < n; i++) { out_r[i] = pe[i].r; out_c[i] = pe[i].c; out_v[i] = pe[i].v; }
    free(le); free(re); free(pe);
    return n;
}

/* Number of OpenMP threads the oracle would use (1 without OpenMP). */
int oracle_max_threads(void)
{
#if defined(_OPENMP)
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n)
{
#if defined(_OPENMP)
    extern void omp_set_num_threads(int);
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
