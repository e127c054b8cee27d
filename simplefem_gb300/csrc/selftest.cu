// Self-test of the bounded device waits. Every wait in the solver kernels (the grid
// barrier of the persistent solvers) gives up after a time limit, records
// FEEC_TIMEOUT and the wait site in the status block, and lets every thread leave, so
// the host gets an error status with the GPU context still usable. This entry point
// exercises that path on purpose and safely: one thread waits, through the same
// wait_counter the grid barrier uses, for a counter value that nothing ever writes,
// with a short limit chosen by the caller; it then returns like a barrier that gave up.
#include <chrono>

#include "feec_device.cuh"
#include "feec_internal.h"
#include "feec_system.h"

namespace feec {
namespace {

__global__ void unset_flag_wait_kernel(DeviceStatus* st, unsigned long long limit_ns) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    // the counter starts at 0 and no thread increments it: the wait can only run out
    wait_counter(st, 1ull, 77, limit_ns);
}

}  // namespace
}  // namespace feec

using namespace feec;

extern "C" int feec_selftest_wait_timeout(double limit_s, int* status, int* site, double* elapsed_ms) {
    if (!(limit_s > 0.0) || limit_s > 10.0) return FEEC_BADARG;
    int dev = 0;
    cudaStream_t lib = nullptr;
    int st = init_device(dev, lib);
    if (st != FEEC_OK) return st;
    DevArena mem;
    mem.stream = lib;
    DeviceStatus* d = nullptr;
    FEEC_TRY(mem.alloc(d, 1));
    FEEC_TRY(cudaMemsetAsync(d, 0, sizeof(DeviceStatus), lib));
    const auto t0 = std::chrono::steady_clock::now();
    note_launch();
    unset_flag_wait_kernel<<<1, 32, 0, lib>>>(d, (unsigned long long)(limit_s * 1e9));
    FEEC_TRY(cudaGetLastError());
    DeviceStatus h{};
    FEEC_TRY(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, lib));
    FEEC_TRY(cudaStreamSynchronize(lib));
    if (elapsed_ms) *elapsed_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    mem.release();
    FEEC_TRY(cudaStreamSynchronize(lib));
    if (status) *status = h.status;
    if (site) *site = h.timeout_site;
    return FEEC_OK;
}
