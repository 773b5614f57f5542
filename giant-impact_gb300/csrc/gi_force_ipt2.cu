// gi_force_ipt2.cu -- force kernel instances with 2 i-bodies per thread.
#include "gi_force_impl.cuh"

cudaError_t gi_launch_force_ipt2(int acc, int epi, const ForceArgs &a,
                                  const LaunchTable &tab, int grid, cudaStream_t s)
{
    return gi::launch_force_ipt<2>(acc, epi, a, tab, grid, s);
}

int gi_force_occupancy_ipt2(int acc, int epi) { return gi::occupancy_ipt<2>(acc, epi); }
