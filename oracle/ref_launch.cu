// ref_launch.cu -- extern "C" launchers around the reference's own kernels.
//
// TEST INFRASTRUCTURE.  The kernels come from the reference sources, cut by
// oracle/build_ref.py into oracle/_ref/*.inc at build time; this file only
// provides the environment they were written for (the includes and
// BLOCKSIZE of Code/CommonCode/commonSetup.h:1-23) and launches them exactly
// as the reference drivers do: <<<N/256, 256>>> on the given stream
// (Code/ImpactCode/impactAddTime.cu:400-401,
// Code/GenerateTargetImpactorCode/generateTargetImpactor.cu:670-711).
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <iostream>
using namespace std;

#define BLOCKSIZE 256

#include "ref_impact_structs.inc"
#include "ref_impact_kernels.inc"
#include "ref_generate_structs.inc"
#include "ref_generate_kernels.inc"

// Status: 0 ok, 2 bad size (the reference needs N % 256 == 0), else the
// cudaError_t of the launch.
extern "C" int giref_forces_collision(const float *pos, const float *vel, float *force,
                                      const void *consts, int n, void *stream)
{
    if (n <= 0 || n % BLOCKSIZE) return 2;
    forceCollisionKernalConstantsStruct c;
    memcpy(&c, consts, sizeof c);
    getForcesCollisionSingleGPU<<<n / BLOCKSIZE, BLOCKSIZE, 0, (cudaStream_t)stream>>>(
        (float4 *)pos, (float4 *)vel, (float4 *)force, c);
    return (int)cudaGetLastError();
}

extern "C" int giref_move_collision(float *pos, float *vel, const float *force,
                                    const void *consts, int n, void *stream)
{
    if (n <= 0 || n % BLOCKSIZE) return 2;
    moveCollisionKernalConstantsStruct c;
    memcpy(&c, consts, sizeof c);
    moveBodiesCollisionSingleGPU<<<n / BLOCKSIZE, BLOCKSIZE, 0, (cudaStream_t)stream>>>(
        (float4 *)pos, (float4 *)vel, (float4 *)force, c);
    return (int)cudaGetLastError();
}

extern "C" int giref_forces_separate(const float *pos, const float *vel, float *force,
                                     const void *consts, int n, void *stream)
{
    if (n <= 0 || n % BLOCKSIZE) return 2;
    forceSeperateKernalConstantsStruct c;
    memcpy(&c, consts, sizeof c);
    getForcesSeperate<<<n / BLOCKSIZE, BLOCKSIZE, 0, (cudaStream_t)stream>>>(
        (float4 *)pos, (float4 *)vel, (float4 *)force, c);
    return (int)cudaGetLastError();
}

extern "C" int giref_move_damped_separate(float *pos, float *vel, const float *force,
                                          const void *consts, float damp1, float damp2,
                                          int n, void *stream)
{
    if (n <= 0 || n % BLOCKSIZE) return 2;
    moveSeperateKernalConstantsStruct c;
    memcpy(&c, consts, sizeof c);
    moveBodiesDampedSeperate<<<n / BLOCKSIZE, BLOCKSIZE, 0, (cudaStream_t)stream>>>(
        (float4 *)pos, (float4 *)vel, (float4 *)force, c, damp1, damp2);
    return (int)cudaGetLastError();
}

extern "C" void giref_struct_sizes(int *out)
{
    out[0] = (int)sizeof(forceCollisionKernalConstantsStruct);
    out[1] = (int)sizeof(moveCollisionKernalConstantsStruct);
    out[2] = (int)sizeof(forceSeperateKernalConstantsStruct);
    out[3] = (int)sizeof(moveSeperateKernalConstantsStruct);
}
