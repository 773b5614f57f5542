// gi_force_ipt1.cu -- force kernel instances with 1 i-bodies per thread, and
// the split-off epilogue (finish_kernel) of GI_EPI_SUM launches.
#include <algorithm>

#include "gi_force_impl.cuh"

cudaError_t gi_launch_force_ipt1(int acc, int epi, const ForceArgs &a,
                                  const LaunchTable &tab, int grid, cudaStream_t s)
{
    return gi::launch_force_ipt<1>(acc, epi, a, tab, grid, s);
}

int gi_force_occupancy_ipt1(int acc, int epi) { return gi::occupancy_ipt<1>(acc, epi); }

cudaError_t gi_launch_finish(int epi, const ForceArgs &a, const LaunchTable &tab, int maxn,
                             int nsm, cudaStream_t s)
{
    if (tab.nruns <= 0 || maxn <= 0) return cudaSuccess;
    const dim3 g((unsigned int)std::min(4 * nsm, (maxn + 255) / 256), (unsigned int)tab.nruns);
    if (epi == GI_EPI_FORCE) gi::finish_kernel<GI_EPI_FORCE><<<g, 256, 0, s>>>(a, tab);
    else if (epi == GI_EPI_STEP) gi::finish_kernel<GI_EPI_STEP><<<g, 256, 0, s>>>(a, tab);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}
