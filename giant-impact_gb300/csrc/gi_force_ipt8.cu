// gi_force_ipt8.cu -- force kernel instances with 8 i-bodies per thread.
#include "gi_force_impl.cuh"

cudaError_t gi_launch_force_ipt8(int acc, int epi, const ForceArgs &a,
                                  const LaunchTable &tab, int grid, cudaStream_t s)
{
    return gi::launch_force_ipt<8>(acc, epi, a, tab, grid, s);
}

int gi_force_occupancy_ipt8(int acc, int epi) { return gi::occupancy_ipt<8>(acc, epi); }
