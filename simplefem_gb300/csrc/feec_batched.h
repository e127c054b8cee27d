// Shared definitions of the batched solver engine (kernels_batched.cu, batched.cu).
#pragma once

#include <cuda_runtime.h>

#include "feec_internal.h"

namespace feec {

constexpr int kBatchMaxK = 8;   // right-hand sides advanced together by one team

// Device view of one system in SELL-32 layout over its color-permuted rows.
struct SellView {
    int n, nslices, ncolors, pad;
    const int* perm;            // permuted row -> caller's row
    const int* slice_row0;      // first permuted row of each slice
    const int* slice_nrow;      // valid rows in each slice (<= 32)
    const int4* slice_len;      // (L, E, U, 0) block lengths of each slice
    const long long* slice_off; // offset of each slice in ci / val
    const int* color_slice;     // slices of color c: [color_slice[c], color_slice[c+1])
    const int* ci;              // column-major blocks, padded entries point at a valid row with value 0
    const float* val32;
    const double* val64;
    const float* wd32; const float* sd32;    // omega / D (0 where D == 0) and D (2 - omega) / omega
    const double* wd64; const double* sd64;
};

struct BatchItem {
    int system;        // index into BatchArgs::systems
    int nrhs;          // columns in use (<= K of the launch)
    int first_result;  // results[first_result + j] receives column j
    int pad;
    const double* b[kBatchMaxK];   // caller right-hand sides (caller numbering)
    double* x[kBatchMaxK];         // caller solutions (caller numbering; in: initial guess)
    double* xp; double* bp; double* r64;                 // n*K FP64 workspace
    void* r; void* d; void* m; void* q; void* c;  // n*K inner workspace (float or double)
};

struct BatchResult {
    int status, iterations, outer;
    int fp64_fallback;        // set on the host when a stagnated column was finished in FP64
    double relres;
    double err_est;           // mixed: estimated relative error of x (-1: not estimated)
};

// Mixed precision, segment by segment: each segment is a fresh FP32 inner solve of the
// residual equation to a fall of kRestartEta (or what the target still needs), after which
// the FP64 true residual is recomputed (plain defect correction). The whole-GPU solver
// keeps the multicolor SSOR-PCG's search direction across replacements after the first
// segment (reliable updates) with segments of kReliableDelta: 3D P2 refined 5 times,
// 39.2 ms against 46.5 restarted. The batched engine restarts: its columns run in
// lockstep, and kept directions gained 2.5 % there. An operator too ill-conditioned for
// FP32 arithmetic shows in the first segment (its true residual gains less than half the
// digits asked) and is finished in FP64. A column gets at most kMaxReplacements segments.
constexpr double kRestartEta = 2e-5;
constexpr double kReliableDelta = 0.01;
// A kept-direction segment may take this many times the iterations per decade of z.r fall
// that the restarted segments of the same solve took (the whole-GPU solver).
constexpr double kKeptSegmentSlack = 2.0;
constexpr int kMaxReplacements = 64;

struct BatchArgs {
    const SellView* systems;
    const BatchItem* items;
    int nitems;
    int* next_item;           // work queue head (zeroed before the launch)
    BatchResult* results;
    double precision;         // stop when ||b - A x|| <= precision ||b|| (FP64)
    double inner_eta;         // segment factor (kRestartEta; 1e-30: only the target)
    int err_control;          // 1: also stop only at the error bar (mixed precision)
    double inner_margin;      // a segment aims at margin * (the residual target)
    int max_iter;             // inner iterations per column, summed over all segments
    int max_outer;            // residual replacements per column
    int stall_check;          // 1: stop a column whose last inner solve gained less than half
                              // the digits asked (status kStatusStagnated; the host finishes it in FP64)
};

// Internal result status of a column stopped by the stall check; never returned to callers.
constexpr int kStatusStagnated = 100;

cudaError_t launch_batched(const BatchArgs& args, int is_float, int K, int rainbow, int threads, int teams,
                           cudaStream_t s);
int batched_resident_teams(int is_float, int K, int rainbow, int threads);
// One request per launch on a cluster of `blocks` thread blocks (kernels_cluster.cu).
cudaError_t launch_cluster(const BatchArgs& args, int item, int is_float, int rainbow, int blocks, cudaStream_t s);
int cluster_max_blocks(int is_float, int rainbow);
int batched_team_threads(int is_float, int requested);
int batched_max_k(int is_float);
// Batched engine with clusters of `blocks` (2..16) thread blocks as teams (kernels_cluster_batched.cu).
cudaError_t launch_batched_clusters(const BatchArgs& args, int is_float, int K, int rainbow, int blocks, int clusters,
                                    cudaStream_t s);
int cluster_batched_resident(int is_float, int K, int rainbow, int blocks);
int cluster_batched_threads();

// y = scaling * A x over a natural-order SELL-32 layout; is_float selects FP32 data
// (x, y float) or FP64 (x, y double). One thread per row, coalesced entry loads.
cudaError_t launch_sell_spmv(const SellView& v, int is_float, const void* x, void* y, double scaling, cudaStream_t s);

// SELL construction (kernels_setup.cu)
cudaError_t launch_sell_lengths(int nslices, const int* slice_row0, const int* slice_nrow, const int* rp,
                                const int* lsplit, const int* usplit, int4* slice_len, cudaStream_t s);
cudaError_t launch_sell_fill(int nslices, const int* slice_row0, const int* slice_nrow, const int4* slice_len,
                             const long long* slice_off, const int* rp, const int* lsplit, const int* usplit,
                             const int* ci_in, const double* val_in, int* ci, float* val32, double* val64,
                             cudaStream_t s);

}  // namespace feec
