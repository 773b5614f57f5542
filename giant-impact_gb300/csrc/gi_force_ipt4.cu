// gi_force_ipt4.cu -- force kernel instances with 4 i-bodies per thread.
#include "gi_force_impl.cuh"

cudaError_t gi_launch_force_ipt4(int acc, int epi, const ForceArgs &a,
                                  const LaunchTable &tab, int grid, cudaStream_t s)
{
    return gi::launch_force_ipt<4>(acc, epi, a, tab, grid, s);
}

int gi_force_occupancy_ipt4(int acc, int epi) { return gi::occupancy_ipt<4>(acc, epi); }
