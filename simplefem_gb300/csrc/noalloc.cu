// Allocation-free plain CG entry point: feec_cg_csr_noalloc.
//
// Some callers cannot allocate device memory while they run a solve: code that
// works inside a fixed memory budget handed out up front (a pool that must not
// grow, a serving process whose device memory is reserved for other work), or
// that runs where a cudaMalloc/cudaFree would synchronise the device or is not
// allowed at all. This entry point lets them call the GPU CG with buffers they
// already own. Its scratch (the search direction, A times it, the per-block
// partial sums and the solver status words) lives in one file-scope device
// array of fixed size, so the call itself allocates nothing.
//
// Limits and sharing rules:
//  * at most kNoAllocMaxRows rows; larger systems are rejected with FEEC_BADARG;
//  * the array is 16 MiB plus a few KiB, and every GPU that loads this library
//    holds it until the process exits;
//  * every call shares the one array and leaves its contents behind: the status
//    words that must start at zero are cleared on each call, and calls whose
//    work overlaps on the GPU (other threads, other streams) race with each
//    other — serialise them;
//  * the first call on a device looks up the array's device address (with that
//    device current) and caches it; make that first call before any stream
//    capture.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "feec_device.cuh"
#include "feec_internal.h"

namespace feec {

constexpr int kNoAllocMaxRows = 1 << 20;       // 1,048,576 rows
constexpr int kNoAllocMaxBlocks = 2048;        // grid size cap (partials sized for it)

struct NoAllocScratch {
    double d[kNoAllocMaxRows];                  // search direction
    double q[kNoAllocMaxRows];                  // A d
    double partials[3 * kNoAllocMaxBlocks + 64];
    DeviceStatus st;
    double bnorm2;
    int bad;
};

// The only storage the entry point uses. In host code this name is a host-side
// stand-in: kernels must be given the address from cudaGetSymbolAddress.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

namespace {

std::mutex g_noalloc_mutex;
NoAllocScratch* g_noalloc_ptr[64] = {};

// Device address of the scratch array on the current device (looked up once per device).
int noalloc_scratch(NoAllocScratch*& out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return FEEC_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return FEEC_CUDA_ERROR;
        g_noalloc_ptr[dev] = (NoAllocScratch*)p;
    }
    out = g_noalloc_ptr[dev];
    return FEEC_OK;
}

int noalloc_cuda(cudaError_t e) { return e == cudaSuccess ? FEEC_OK : FEEC_CUDA_ERROR; }

}  // namespace
}  // namespace feec

using namespace feec;

extern "C" int feec_cg_csr_noalloc(int N, double* x, const double* b, const int* A, const int* C, const double* V,
                                   double* residual, double precision, int max_iter, feec_solve_info* info,
                                   void* stream) {
    if (info) {
        *info = feec_solve_info{};
        info->true_relres = -1.0;
        info->outer_iterations = 1;
        info->error_estimate = -1.0;
    }
    // every early return records its code in info->status as well
    auto fail = [info](int code) {
        if (info) info->status = code;
        return code;
    };
    if (N <= 0 || !x || !b || !A || !C || !V || !residual || !(precision > 0.0)) return fail(FEEC_BADARG);
    if (N > kNoAllocMaxRows) {
        std::fprintf(stderr, "feec_cg_csr_noalloc: N = %d exceeds the fixed scratch capacity of %d rows\n", N,
                     kNoAllocMaxRows);
        return fail(FEEC_BADARG);
    }
    NoAllocScratch* sc = nullptr;
    int st = noalloc_scratch(sc);
    if (st != FEEC_OK) return fail(st);
    cudaStream_t s = (cudaStream_t)stream;

    // structural check of the caller's CSR before any kernel indexes through it
    int nnz = -1;
    cudaError_t e = cudaMemcpyAsync(&nnz, A + N, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(noalloc_cuda(e));
    if (nnz < 0) return fail(FEEC_BADARG);
    int bad = 0;
    if ((e = cudaMemsetAsync(&sc->bad, 0, sizeof(int), s)) != cudaSuccess ||
        (e = launch_validate_csr(N, nnz, A, C, &sc->bad, s)) != cudaSuccess ||
        (e = launch_sum_sq_f64(N, b, &sc->bnorm2, s)) != cudaSuccess)
        return fail(noalloc_cuda(e));
    double bnorm2 = 0.0;
    if ((e = cudaMemcpyAsync(&bad, &sc->bad, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&bnorm2, &sc->bnorm2, sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail(noalloc_cuda(e));
    if (bad) return fail(FEEC_BADARG);

    // tolerance exactly as solver/sparsesolver.cpp:45-48 (norm summed on the device)
    const double kFloor = 1.490116119384765625e-08;
    double tolerance = precision * std::sqrt(bnorm2);
    if (!(tolerance >= kFloor)) tolerance = tolerance != tolerance ? tolerance : kFloor;

    // the status words (barrier counter, abort flag, status) must start at zero
    if ((e = cudaMemsetAsync(&sc->st, 0, sizeof(DeviceStatus), s)) != cudaSuccess) return fail(noalloc_cuda(e));

    CgArgs<double> a{};
    a.n = N; a.rp = A; a.ci = C; a.val = V; a.b = b; a.x = x; a.r = residual; a.d = sc->d; a.q = sc->q;
    a.tol2 = tolerance * tolerance;
    a.max_iter = max_iter > 0 ? max_iter : N;
    a.print_modulo = -3;
    a.print_tol = tolerance;
    a.partials = sc->partials;
    a.st = &sc->st;
    LaunchShape shape;
    shape.lanes = pick_lanes((double)nnz / (double)N);
    shape.threads = 512;
    const int maxb = max_coresident_blocks(0, 0, shape.lanes, shape.threads);
    if (maxb > kNoAllocMaxBlocks) shape.blocks = kNoAllocMaxBlocks;
    if ((e = launch_cg<double>(a, shape, s)) != cudaSuccess) return fail(noalloc_cuda(e));
    DeviceStatus hs{};
    if ((e = cudaMemcpyAsync(&hs, &sc->st, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail(noalloc_cuda(e));
    if (info) {
        info->status = hs.status;
        info->iterations = hs.iterations;
        info->tolerance = tolerance;
        info->final_norm = std::sqrt(std::fabs(hs.final_value));
        info->grid_blocks = shape.blocks;
        info->lanes_per_row = shape.lanes;
    }
    return hs.status;
}
