// Batched solver engine: one thread block ("team") per work item, a work item
// being K right-hand sides of one system advanced in lockstep. Teams never wait
// on each other, so the launch needs no co-residency and every phase barrier is
// a block barrier. Each team runs a complete solve:
//
//   FP64 defect correction (outer):  r = b - A x in FP64, stop on ||r|| / ||b||
//   inner PCG (T = float: mixed mode, T = double: FP64 mode) on A c = r / ||r||,
//   with the reference's multicolor SSOR sweeps (ConjugateGradientSolverCSR_Rainbow,
//   solver/sparsesolver.cpp:1002-1335) or no preconditioner (plain CG, :26-201),
//   then x += ||r|| c.
//
// Matrix layout: SELL-32 ("sliced ELL") over the color-permuted rows. A slice is 32
// consecutive rows of one color; its entries are stored column-major in three
// blocks [L | E | U] (colors lower / equal / higher than the row's), each padded to
// the slice's longest row with zero entries. A warp owns a slice, a thread owns a
// row: loads of column indices and values are fully coalesced, no cross-lane
// reduction is needed, and the per-row epilogue runs on all lanes at once.
// Vectors of a team are interleaved [row][K] so one gather fetches the K values
// of a column in a single 8/16/32-byte load.
#include "team_solver.cuh"

namespace feec {
namespace {

using namespace team_solver;

// At least 1024 resident threads per SM (64 registers per thread): the solver is bound by
// memory latency, so warps in flight matter more than registers.
template <typename T, int K, bool RAINBOW, int THREADS>
__global__ void __launch_bounds__(THREADS, (1024 / THREADS) > 0 ? (1024 / THREADS) : 1) batched_solve_kernel(BatchArgs args) {
    __shared__ int s_item;
    while (true) {
        if (threadIdx.x == 0) s_item = atomicAdd(args.next_item, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= args.nitems) return;
        BlockTeam team;
        team_solve<T, K, RAINBOW>(team, args, args.items[item]);
    }
}

template <typename T, int K, bool RB>
const void* kfn(int threads) {
    if constexpr (sizeof(T) == 4 && K == 8) {
        if (threads == 512) return (const void*)batched_solve_kernel<T, K, RB, 512>;
        return (const void*)batched_solve_kernel<T, K, RB, 256>;
    }
    if constexpr (sizeof(T) == 4 && K < 8) {
        if (threads == 128) return (const void*)batched_solve_kernel<T, K, RB, 128>;
        if (threads == 512) return (const void*)batched_solve_kernel<T, K, RB, 512>;
        if constexpr (K <= 2) {
            if (threads == 1024) return (const void*)batched_solve_kernel<T, K, RB, 1024>;
        }
    }
    return (const void*)batched_solve_kernel<T, K, RB, 256>;
}

// nullptr for a (precision, K) without a compiled kernel: a work item's vectors are laid out
// for its K, so a kernel of another K must never run it.
const void* pick(int is_float, int K, int rainbow, int threads) {
    if (is_float) {
        switch (K) {
            case 1: return rainbow ? kfn<float, 1, true>(threads) : kfn<float, 1, false>(threads);
            case 2: return rainbow ? kfn<float, 2, true>(threads) : kfn<float, 2, false>(threads);
            case 4: return rainbow ? kfn<float, 4, true>(threads) : kfn<float, 4, false>(threads);
            case 8: return rainbow ? kfn<float, 8, true>(threads) : kfn<float, 8, false>(threads);
            default: return nullptr;
        }
    }
    switch (K) {
        case 1: return rainbow ? kfn<double, 1, true>(threads) : kfn<double, 1, false>(threads);
        case 2: return rainbow ? kfn<double, 2, true>(threads) : kfn<double, 2, false>(threads);
        default: return nullptr;
    }
}

}  // namespace

int batched_max_k(int is_float) { return is_float ? 8 : 2; }

int batched_team_threads(int is_float, int requested) {
    if (!is_float) return 256;
    return (requested == 128 || requested == 512 || requested == 1024) ? requested : 256;
}

// The block size of the kernel that runs (K = 8 exists for 256 and 512 threads only).
int team_threads_for(int is_float, int K, int requested) {
    const int t = batched_team_threads(is_float, requested);
    return (K == 8 && t != 512) ? 256 : t;
}

int batched_resident_teams(int is_float, int K, int rainbow, int threads) {
    threads = team_threads_for(is_float, K, threads);
    const void* fn = pick(is_float, K, rainbow, threads);
    if (!fn) return 0;
    const int smem = team_dynamic_smem(threads);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem);
    return sms * (per > 0 ? per : 1);
}

cudaError_t launch_batched(const BatchArgs& args, int is_float, int K, int rainbow, int threads, int teams, cudaStream_t s) {
    threads = team_threads_for(is_float, K, threads);
    const void* fn = pick(is_float, K, rainbow, threads);
    if (!fn) return cudaErrorInvalidValue;
    const int smem = team_dynamic_smem(threads);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    if (teams <= 0) teams = batched_resident_teams(is_float, K, rainbow, threads);
    if (teams > args.nitems) teams = args.nitems;
    if (teams <= 0) return cudaSuccess;
    BatchArgs copy = args;
    void* kargs[] = {&copy};
    note_launch();
    return cudaLaunchKernel(fn, dim3(teams), dim3(threads), kargs, (size_t)smem, s);
}

}  // namespace feec
