// The device-resident system object and small host helpers shared by the
// C ABI translation units (capi.cu, batched.cu).
#pragma once

#include <cstddef>
#include <vector>

#include <cuda_runtime.h>

#include "feec_batched.h"
#include "feec_internal.h"

namespace feec {

inline int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return FEEC_OK;
    if (e == cudaErrorMemoryAllocation) return FEEC_OOM;
    return FEEC_CUDA_ERROR;
}

// Stream-ordered device allocations owned by one object.
struct DevArena {
    std::vector<void*> ptrs;
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
    template <typename T>
    cudaError_t alloc(T*& p, size_t count) {
        p = nullptr;
        if (count == 0) count = 1;
        void* q = nullptr;
        cudaError_t e = cudaMallocAsync(&q, count * sizeof(T), stream);
        if (e != cudaSuccess) return e;
        ptrs.push_back(q);
        bytes += count * sizeof(T);
        p = (T*)q;
        return cudaSuccess;
    }
    void release() {
        for (void* p : ptrs) cudaFreeAsync(p, stream);
        ptrs.clear();
        bytes = 0;
    }
};

#define FEEC_TRY(expr)                                        \
    do {                                                      \
        cudaError_t _e = (expr);                              \
        if (_e != cudaSuccess) return ::feec::cuda_status(_e); \
    } while (0)

int init_device(int& dev, cudaStream_t& stream);

// While alive, routes a system's work to its creation ("home") stream, after the
// stream of the current call has drained; used for one-time set-up whose
// allocations outlive the call (their frees are ordered on the home stream).
struct HomeStreamScope;

// A SELL-32 copy of a system's matrix (see SellView).
struct SellData {
    DevArena mem;
    bool ready = false;
    int nslices = 0, ncolors = 0;
    int* slice_row0 = nullptr; int* slice_nrow = nullptr; int4* slice_len = nullptr; long long* slice_off = nullptr;
    int* color_slice = nullptr; int* ci = nullptr; float* val32 = nullptr; double* val64 = nullptr;
    int* ident = nullptr;
    long long entries = 0;
};

}  // namespace feec

struct feec_system {
    int dev = 0;
    int n = 0;
    int nnz = 0;
    cudaStream_t stream = nullptr;         // stream of the current call
    cudaStream_t home_stream = nullptr;    // stream given at creation: owns every persistent allocation
    feec::DevArena mem;      // matrix + layouts
    feec::DevArena work;     // Krylov workspace
    int* A = nullptr; int* C = nullptr; double* V = nullptr;   // original CSR
    float* V32 = nullptr;                                        // FP32 copy for mixed CG
    int lanes = 4;
    // preconditioner layout (valid if prepared >= 0)
    int prepared = -1;
    int* perm = nullptr; int* iperm = nullptr;
    int* rp = nullptr; int* ci = nullptr; double* val = nullptr; float* val32 = nullptr;
    int* lsplit = nullptr; int* usplit = nullptr;
    double* diag = nullptr; float* diag32 = nullptr;
    double* wd = nullptr; double* sd = nullptr; float* wd32 = nullptr; float* sd32 = nullptr;
    int nf = 0; int* fptr = nullptr;
    int nbw = 0; int* bptr = nullptr; int* brows = nullptr;
    int* fsplit = nullptr; int* bsplit = nullptr;   // multicolor: end of each phase's long rows
    double omega = 1.0;
    int num_levels = 0;
    // workspace (FP64 permuted vectors + FP32 inner vectors)
    bool work_ready = false;
    double *x = nullptr, *r = nullptr, *d = nullptr, *z = nullptr, *m = nullptr, *q = nullptr, *b = nullptr;
    double* w = nullptr;               // Eisenstat solvers only: auxiliary + technical
    float* w32 = nullptr;              // ... FP32 copy for the mixed-precision inner solves
    char* sweep_rec = nullptr;         // one-block solver: per-row sweep records (both sweeps)
    // MIXED on the whole GPU, per method slot (0: plain CG, 1: preconditioned): 0 = not yet
    // measured, 1 = FP32 inner iterations, 2 = FP64; device ms per decade of residual fall
    int mixed_pick[2] = {0, 0};
    double mixed_rate[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    int zero_diag_rows = 0;            // rows with D == 0 in the prepared layout (the sweeps skip them)
    double* precon = nullptr;          // diagonal preconditioner of FEEC_METHOD_DIAGONAL (original numbering)
    float *x32 = nullptr, *r32 = nullptr, *d32 = nullptr, *z32 = nullptr, *m32 = nullptr, *q32 = nullptr, *b32 = nullptr;
    double* partials = nullptr;
    double* scal = nullptr;   // device scalars
    feec::DeviceStatus* st = nullptr;
    int max_blocks = 0;
    int max_phase_rows = 0;     // largest sweep phase (rows)
    int user_blocks = 0;        // launch-shape overrides (0 = automatic)
    int user_lanes = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // SELL-32 layouts: [0] natural row order (SpMV, batched plain CG), [1] Rainbow order
    feec::SellData sell[2];
    // batched-engine launch choice made by the autotuner, per [method][mode] (0 = not tuned)
    int tuned_k[3][3] = {};
    int tuned_threads[3][3] = {};
    int tuned_blocks[3][3] = {};       // blocks per team: 1 = block team, 2..16 = cluster team
    double tuned_rate[3][3] = {};
};

namespace feec {
struct HomeStreamScope {
    feec_system* s;
    cudaStream_t saved;
    explicit HomeStreamScope(feec_system* sys) : s(sys), saved(sys->stream) {
        if (saved != s->home_stream) {
            cudaStreamSynchronize(saved);
            s->stream = s->home_stream;
        }
    }
    ~HomeStreamScope() {
        if (saved != s->home_stream) {
            cudaStreamSynchronize(s->home_stream);
            s->stream = saved;
        }
    }
};
}  // namespace feec
