// Internal interfaces between the host orchestration (capi.cu), the persistent
// solver kernels (kernels_krylov.cu), the layout/SpMV kernels (kernels_setup.cu)
// and the host integer preprocessing (coloring.cpp).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "feec_gpu.h"

namespace feec {

struct DeviceStatus;

// Mixed precision stops only when its estimated relative solution error is at most this
// many times the requested relative residual (1e-9 at a request of 1e-10).
constexpr double kErrorPerResidual = 10.0;
// The amplification assumed until a larger one is measured: the stopping residual is at most
// kErrorPerResidual x precision / max(measured amplification, kAmpFloor). Measured on the
// benchmark operators (2D P2, 3D P1 and P2, 4,913 to 2.1 M unknowns), the final error of a
// mixed solve was at most 43 times its relative residual.
constexpr double kAmpFloor = 100.0;

// ---------------------------------------------------------------------------
// Persistent solver arguments (all pointers are device pointers).
// ---------------------------------------------------------------------------
template <typename T>
struct CgArgs {
    int n;
    const int* rp; const int* ci; const T* val;
    const T* b;
    T* x; T* r; T* d; T* q;
    double tol2;        // stop when r.r < tol2 (reference rule) ...
    int max_iter;       // ... or after max_iter iterations
    int print_modulo;
    double print_tol;   // tolerance printed in interim lines
    double* partials;   // >= 3 * gridDim.x doubles
    DeviceStatus* st;
    // diagonal preconditioner (ConjugateGradientSolverCSR_DiagonalPreconditioner) when not
    // null: z = precon * r, rows with precon == 0 are skipped, the stop test is on z.r
    const T* precon;
    T* z;
    // reliable updates of the mixed-precision solver: keep_dir = 1 keeps the search
    // direction d of the previous segment, forming d = r + beta d with beta =
    // r.r / (zr_prev * scale) after the restart (scale = old over new residual scale);
    // the kernel leaves its last rho_prev in st->extra[0]
    int keep_dir;
    double zr_prev, scale;
    // one-block solver with one-warp sweeps (kernels_small.cu): per-row sweep records in
    // forward and backward sweep order, built by launch_build_sweep_records
    const void* sweep_fwd;
    const void* sweep_bwd;
};

template <typename T>
struct PcgArgs {
    int n;
    const int* rp; const int* ci; const T* val;   // rows ordered [L | E | U]
    const int* lsplit; const int* usplit;         // L = [rp, lsplit), E = [lsplit, usplit), U = [usplit, rp+1)
    const T* wd; const T* sd;                     // omega / D (0 where D == 0) and D (2 - omega) / omega
    const T* b;
    T* x; T* r; T* d; T* z; T* m; T* q;
    int nf; const int* fptr;                      // forward phases: rows [fptr[p], fptr[p+1])
    int nbw; const int* bptr; const int* brows;   // backward phases: rows brows[bptr[p] .. bptr[p+1])
    // multicolor layouts (rows of a color longest first): the long rows of forward phase p
    // are [fptr[p], fsplit[p]), of backward phase p the slots [bptr[p], bsplit[p]); null otherwise
    const int* fsplit; const int* bsplit;
    double omega;
    double tol2;         // reference rule: stop when |z.r| < tol2 (if use_zr_rule)
    double rr_stop;      // stop when the recursive r.r < rr_stop (if > 0); Eisenstat: when z.r < rr_stop * (z.r at the start)
    int use_zr_rule;
    int max_iter;
    int print_modulo;
    double print_tol;
    double* partials;    // >= 3 * gridDim.x doubles
    DeviceStatus* st;
    // Eisenstat variants only
    const T* dg;         // the diagonal D, permuted like the rows
    T* w;                // the sweeps' combined vector (auxiliary + technical)
    int guard_restart;   // skip entries whose column has D == 0 in the restart sweeps
    int guard_iter;      // ... and in the iteration sweeps (index-order variant)
    // reliable updates (Eisenstat kernel, mixed precision): keep_dir = 1 keeps the direction d
    // of the previous segment (d = z + beta d with beta = z.r / (zr_prev * scale) after the
    // restart); the kernel leaves its last rho_prev in st->extra[0]
    int keep_dir;
    double zr_prev, scale;
    // one-block solver with one-warp sweeps (kernels_small.cu): per-row sweep records in
    // forward and backward sweep order, built by launch_build_sweep_records
    const void* sweep_fwd;
    const void* sweep_bwd;
};

// Rows with more stored entries than this count as long in a multicolor layout: the
// persistent sweeps give them more lanes (the phase bounds fsplit / bsplit).
constexpr int kLongRowEntries = 32;

struct LaunchShape {
    int blocks = 0;
    int threads = 0;
    int lanes = 0;
};

// Kernel launchers (kernels_krylov.cu). Return the CUDA error of the launch.
template <typename T> cudaError_t launch_cg(const CgArgs<T>& a, LaunchShape& shape, cudaStream_t s);
template <typename T> cudaError_t launch_pcg(const PcgArgs<T>& a, LaunchShape& shape, cudaStream_t s);
// SSOR-PCG with Eisenstat's trick over the same phase schedules (kernels_eisenstat.cu).
template <typename T> cudaError_t launch_eisenstat(const PcgArgs<T>& a, LaunchShape& shape, cudaStream_t s);
// FP64 SSOR / multicolor SSOR PCG in one block with the gathered vectors in shared memory
// (kernels_small.cu), for systems of at most pcg_smem_max_rows() rows.
cudaError_t launch_pcg_smem(const PcgArgs<double>& a, int lanes, int threads, cudaStream_t s);
int pcg_smem_max_rows();
int pcg_smem_threads(int max_phase_rows, int lanes);
bool pcg_smem_warp_sweeps(int n, int nf, int nbw);   // one warp walks the sweeps (256-thread block)
size_t sweep_record_bytes(int n);                   // both sweeps' records of an n-row system
cudaError_t launch_build_sweep_records(const PcgArgs<double>& a, void* recs, cudaStream_t s);
// Largest co-resident grid for the given kernel family and lane count.
int max_coresident_blocks(int family, int is_float, int lanes, int threads);
int pick_lanes(double avg_nnz_per_row);

// Setup / utility kernels (kernels_setup.cu).
cudaError_t launch_spmv_f64(int n, const int* rp, const int* ci, const double* v, const double* x, double* y,
                            double scaling, int lanes, cudaStream_t s);
cudaError_t launch_residual_f64(int n, const int* rp, const int* ci, const double* v, const double* b,
                                const double* x, double* r, double* partial_sq, int lanes, cudaStream_t s);
cudaError_t launch_sum_sq_f64(int n, const double* v, double* out, cudaStream_t s);
cudaError_t launch_permute_split(int n, const int* A, const int* C, const double* V, const int* perm,
                                 const int* iperm, const int* key, const int* new_rp, int* out_ci,
                                 double* out_v, float* out_v32, int* lsplit, int* usplit, cudaStream_t s);
cudaError_t launch_validate_csr(int n, int nnz, const int* A, const int* C, int* bad, cudaStream_t s);
// rows x ncols: row pointers monotone from 0 to nnz, columns in [0, ncols); sets *bad on a violation
cudaError_t launch_validate_csr_cols(int n, int ncols, int nnz, const int* A, const int* C, int* bad, cudaStream_t s);
cudaError_t launch_row_lengths(int n, const int* A, const int* perm, int* len, cudaStream_t s);
cudaError_t launch_exclusive_scan(int n, const int* in, int* out, int* scratch, cudaStream_t s);
cudaError_t launch_inverse_perm(int n, const int* perm, int* iperm, cudaStream_t s);
cudaError_t launch_gather_f64(int n, const int* perm, const double* src, double* dst, cudaStream_t s);
cudaError_t launch_scatter_f64(int n, const int* perm, const double* src, double* dst, cudaStream_t s);
cudaError_t launch_gather_to_f32(int n, const int* perm, const double* src, float* dst, cudaStream_t s);
cudaError_t launch_diagonal_f64(int n, const int* A, const int* C, const double* V, double* d, cudaStream_t s);
cudaError_t launch_cast_f64_f32(size_t n, const double* src, float* dst, cudaStream_t s);
cudaError_t launch_sweep_factors(int n, const double* diag, double omega, double* wd, double* sd, float* wd32,
                                 float* sd32, cudaStream_t s);
// Mixed precision helpers.
cudaError_t launch_scaled_cast(int n, const double* r, const double* inv_norm_dev, float* r32, cudaStream_t s);
cudaError_t launch_update_x(int n, const int* perm, const float* c32, const double* norm_dev, double* x, cudaStream_t s);
// x += (*norm_dev) c32 (unpermuted) and out2[0] = ||correction||^2, out2[1] = ||x||^2
// (deterministic: per-block partials in `partials`, at least update_norm_blocks(n) x 2)
cudaError_t launch_update_x_norms(int n, const float* c32, const double* norm_dev, double* x, double* partials,
                                  double* out2, cudaStream_t s);
int update_norm_blocks(int n);
void note_launch();

// Host integer preprocessing (coloring.cpp).
int rainbow_host(int n, const int* A, const int* C, int* F, int* B, int* R);
// Level schedule of the strictly lower (forward) or upper (backward) triangle in
// index order: level[i] = 1 + max(level of earlier-solved neighbours).
void triangular_levels(int n, const int* A, const int* C, bool lower, std::vector<int>& level, int& nlevels);

size_t scan_scratch_ints(int n);

}  // namespace feec
