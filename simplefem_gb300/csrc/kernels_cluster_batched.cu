// Batched clusters: the batched engine with a thread-block cluster (2 to 16 blocks)
// as the team. Every cluster takes work items (K right-hand sides of one system)
// from the queue until none are left and solves each with all of its blocks —
// cluster barriers between dependent phases, team sums over distributed shared
// memory. A batch with fewer work items than the GPU holds block teams (64
// right-hand sides of one 66k-row system: 16 items of 4) then still fills the
// SMs. Clusters never wait on each other, so the launch needs no co-residency
// beyond a cluster's own blocks, which the hardware schedules together.
#include <cooperative_groups.h>

#include "team_solver.cuh"

namespace feec {
namespace {

using namespace team_solver;

constexpr int kTeamThreads = 512;

template <typename T, int K, bool RAINBOW>
__global__ void __launch_bounds__(kTeamThreads, 1024 / kTeamThreads) cluster_batched_kernel(BatchArgs args) {
    __shared__ int s_item;
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    while (true) {
        if (cl.block_rank() == 0 && threadIdx.x == 0) s_item = atomicAdd(args.next_item, 1);
        cl.sync();
        const int item = *cl.map_shared_rank(&s_item, 0);
        cl.sync();   // every block has read rank 0's slot before the next item overwrites it
        if (item >= args.nitems) return;
        ClusterTeam team;
        team_solve<T, K, RAINBOW>(team, args, args.items[item]);
        team.sync();   // distributed shared memory of every block stays valid until all are done
    }
}

// nullptr for a K without a compiled kernel (a work item's vectors are laid out for its K).
template <typename T, bool RB>
const void* kfn(int K) {
    if constexpr (sizeof(T) == 4) {
        if (K == 8) return (const void*)cluster_batched_kernel<T, 8, RB>;
        if (K == 4) return (const void*)cluster_batched_kernel<T, 4, RB>;
    }
    if (K == 2) return (const void*)cluster_batched_kernel<T, 2, RB>;
    if (K == 1) return (const void*)cluster_batched_kernel<T, 1, RB>;
    return nullptr;
}

const void* pick(int is_float, int K, int rainbow) {
    if (is_float) return rainbow ? kfn<float, true>(K) : kfn<float, false>(K);
    return rainbow ? kfn<double, true>(K) : kfn<double, false>(K);
}

cudaLaunchConfig_t cluster_config(int blocks, int clusters, cudaLaunchAttribute& attr, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.dynamicSmemBytes = team_dynamic_smem(kTeamThreads);
    cfg.gridDim = dim3(blocks * clusters);
    cfg.blockDim = dim3(kTeamThreads);
    cfg.stream = s;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = blocks; attr.val.clusterDim.y = 1; attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return cfg;
}

cudaError_t prepare(const void* fn, int blocks) {
    if (blocks > 8) {
        const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, team_dynamic_smem(kTeamThreads));
}

}  // namespace

int cluster_batched_threads() { return kTeamThreads; }

int cluster_batched_resident(int is_float, int K, int rainbow, int blocks) {
    if (blocks < 2 || blocks > 16) return 0;
    const void* fn = pick(is_float, K, rainbow);
    if (!fn || prepare(fn, blocks) != cudaSuccess) return 0;
    cudaLaunchAttribute attr;
    cudaLaunchConfig_t cfg = cluster_config(blocks, 1, attr, nullptr);
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) return 0;
    return n;
}

cudaError_t launch_batched_clusters(const BatchArgs& args, int is_float, int K, int rainbow, int blocks, int clusters,
                                    cudaStream_t s) {
    const void* fn = pick(is_float, K, rainbow);
    if (!fn) return cudaErrorInvalidValue;
    cudaError_t e = prepare(fn, blocks);
    if (e != cudaSuccess) return e;
    if (clusters <= 0) clusters = cluster_batched_resident(is_float, K, rainbow, blocks);
    if (clusters > args.nitems) clusters = args.nitems;
    if (clusters <= 0) return cudaErrorInvalidConfiguration;
    cudaLaunchAttribute attr;
    cudaLaunchConfig_t cfg = cluster_config(blocks, clusters, attr, s);
    BatchArgs copy = args;
    void* kargs[] = {&copy};
    note_launch();
    return cudaLaunchKernelExC(&cfg, fn, kargs);
}

}  // namespace feec
