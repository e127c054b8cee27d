// Cluster engine: one thread-block cluster (1 to 16 blocks, co-scheduled by the
// hardware) solves one request from start to finish — the same device solver as
// the batched engine, with cluster barriers between dependent phases and team sums
// over distributed shared memory. Each launch is independent of every other launch,
// so requests on different streams overlap freely on the GPU; no thread ever waits
// on work outside its own cluster.
#include "team_solver.cuh"

namespace feec {
namespace {

using namespace team_solver;

constexpr int kClusterThreads = 512;

template <typename T, bool RAINBOW>
__global__ void __launch_bounds__(kClusterThreads, 1024 / kClusterThreads) cluster_solve_kernel(BatchArgs args, int item) {
    ClusterTeam team;
    team_solve<T, 1, RAINBOW>(team, args, args.items[item]);
    team.sync();   // distributed shared memory of every block stays valid until all are done
}

const void* cluster_fn(int is_float, int rainbow) {
    if (is_float) return rainbow ? (const void*)cluster_solve_kernel<float, true> : (const void*)cluster_solve_kernel<float, false>;
    return rainbow ? (const void*)cluster_solve_kernel<double, true> : (const void*)cluster_solve_kernel<double, false>;
}

}  // namespace

int cluster_max_blocks(int is_float, int rainbow) {
    const void* fn = cluster_fn(is_float, rainbow);
    cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    const int smem = team_dynamic_smem(kClusterThreads);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaLaunchConfig_t cfg = {};
    cfg.dynamicSmemBytes = smem;
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(kClusterThreads);
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = 16; attr.val.clusterDim.y = 1; attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int sz = 0;
    if (cudaOccupancyMaxPotentialClusterSize(&sz, fn, &cfg) != cudaSuccess) return 8;
    return sz > 0 ? sz : 1;
}

cudaError_t launch_cluster(const BatchArgs& args, int item, int is_float, int rainbow, int blocks, cudaStream_t s) {
    const void* fn = cluster_fn(is_float, rainbow);
    if (blocks > 8) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    const int smem = team_dynamic_smem(kClusterThreads);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.dynamicSmemBytes = smem;
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = blocks; attr.val.clusterDim.y = 1; attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    BatchArgs copy = args;
    void* kargs[] = {&copy, &item};
    note_launch();
    return cudaLaunchKernelExC(&cfg, fn, kargs);
}

}  // namespace feec
