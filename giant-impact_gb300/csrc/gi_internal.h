// gi_internal.h -- device-side tables and launch plumbing shared by the
// libgi translation units.  Not part of the public ABI (see include/gi_api.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gi_api.h"

// Threads per CTA of the one-sided force kernel (gi_force_impl.cuh); also
// its j-tile staged in shared memory and the granularity of its Kahan fold
// (one fold per 128 j).  The paired far field's shape is kPair* below.
#define GI_NT 128
// Runs and pair tables carried by value in one launch.
#define GI_MAX_RUNS 64
#define GI_MAX_PARAMS 8
// Padding position for j beyond a chunk / i beyond a run: far enough that
// gravity underflows to zero, never within contact range of a real body.
#define GI_FAR_J 1.0e16f
#define GI_FAR_I (-1.0e16f)

#define GI_ACC_PAIRED GI_ACCUM_PAIRED  // gi_force_pair.cu
#define GI_ACC_KAHAN GI_ACCUM_KAHAN    // the one-sided kernel's modes
#define GI_ACC_FP32 GI_ACCUM_FP32
#define GI_ACC_FP64 GI_ACCUM_FP64

#define GI_EPI_FORCE 0  // write force[i].xyz
#define GI_EPI_STEP 1   // fused kick-drift into the other state buffer
#define GI_EPI_SUM 2    // FP64 far-field sums into fsum; gi_launch_finish completes

// Pair constants indexed by the pair class test = (i is Fe) + (j is Fe):
// 0 = Si-Si, 1 = Fe-Si, 2 = Fe-Fe.
struct PairDev {
    double fx_unit;      // fixed-point unit of the contact corrections (force)
    float gm_fe, gm_si;  // sqrt(G) m: G m_i m_j = gm_i gm_j (far-field gravity)
    float G[3];          // G m_i m_j of the class (contact band)
    float K[3];          // full stiffness
    float KRmid[3];      // reduced stiffness, middle shell band (Fe-Si: KRMix)
    float KRin[3];       // reduced stiffness, inner band
    float Tband[3];      // r >= ShellBreak(1)  <=>  r2 >= Tband
    float Tmid[3];       // r >= ShellBreakFeSi2 <=> r2 >= Tmid (= Tband otherwise)
    float inv_unit;      // (float)(1 / fx_unit), the scale of a pair term into fixed point
};

struct RunDev {
    int offset, n, nfe, param;
    int item_start;   // first work item of this run
    int nsplit;       // j-chunks per i-block
    int jchunk;       // bodies per big chunk (GI_NT * 2^lg)
    int nib;          // i-blocks
    int lg;           // log2 of the big chunk in tiles of GI_NT bodies
    int tiles;        // tiles of the run, ceil(n / GI_NT)
    int tick_base;    // first ticket of this run
    long long part_base;  // first double of this run's partial sums
    float dt, dtm_fe, dtm_si, damp;
    int ipt;          // i-bodies per thread this run was planned for
    // GI_ACC_PAIRED decomposition (gi_force_pair.cu)
    int pcl;          // log2 of the j-chunks per work item
    int pnc;          // j-chunks of the run, ceil(n / kPairChunk)
    int pnb;          // i-blocks of the run, ceil(n / kPairRows)
    int pk0;          // work items of i-block 0, ceil(pnc / 2^pcl)
    int pitems;       // work items of the run
    int pstride;      // CTA t of the run takes item (t * pstride) mod pitems (coprime)
    float far_inv;    // 1 / far_unit: scale of a far-field sum into fixed point
    double far_unit;  // fixed-point unit of the far-field sums (a power of two)
};

struct LaunchTable {
    int nruns;
    int nitems;
    int sep_test;
    int dense_min;  // contact pass: bucket size from which the tiled kernel takes it
    RunDev runs[GI_MAX_RUNS];
    PairDev params[GI_MAX_PARAMS];
};

struct ForceArgs {
    const float4 *pos;
    const float4 *vel;
    float4 *force;     // GI_EPI_FORCE
    float4 *pos_out;   // GI_EPI_STEP
    float4 *vel_out;   // GI_EPI_STEP
    double *partials;  // split-j partial sums (nullptr when no run splits)
    unsigned int *tickets;
    unsigned int *queue;  // [0] next work item, [1] CTAs finished (zero between launches)
    const long long *delta;  // contact corrections, 3 per body, fixed point (gi_grid.cu)
    double *fsum;            // GI_EPI_SUM: far-field sums, 3 per body
    long long *fsum_fx;      // GI_ACC_PAIRED: far-field sums, 3 per body, fixed point
};

// Launchers (gi_force_ipt*.cu).  Return cudaError_t of the launch.
cudaError_t gi_launch_force(int ipt, int acc, int epi, const ForceArgs &a,
                            const LaunchTable &tab, int grid, cudaStream_t s);
cudaError_t gi_launch_force_ipt1(int acc, int epi, const ForceArgs &a, const LaunchTable &tab, int grid, cudaStream_t s);
cudaError_t gi_launch_force_ipt2(int acc, int epi, const ForceArgs &a, const LaunchTable &tab, int grid, cudaStream_t s);
cudaError_t gi_launch_force_ipt4(int acc, int epi, const ForceArgs &a, const LaunchTable &tab, int grid, cudaStream_t s);
cudaError_t gi_launch_force_ipt8(int acc, int epi, const ForceArgs &a, const LaunchTable &tab, int grid, cudaStream_t s);
// Resident CTAs per SM of a force kernel instance (for the planner).
int gi_force_occupancy(int ipt, int acc, int epi);
// The epilogue of a GI_EPI_SUM launch (epi = GI_EPI_FORCE or GI_EPI_STEP):
// adds the contact corrections and stores or steps, one thread per body.
cudaError_t gi_launch_finish(int epi, const ForceArgs &a, const LaunchTable &tab, int maxn,
                             int nsm, cudaStream_t s);

// gi_force_pair.cu: the far field with each unordered pair evaluated once.
// Its shape is fixed here, where the planner reads it.
namespace gi {
constexpr int kPairWarps = 4;                             // warps per CTA
constexpr int kPairIpl = 8;                               // i-bodies per lane
constexpr int kPairWarpRows = 32 * kPairIpl;              // 256 rows per warp
constexpr int kPairRows = kPairWarps * kPairWarpRows;     // 1024: the i-block
constexpr int kPairChunk = 64;                            // j-chunk: two bodies per lane
constexpr int kPairBlockChunks = kPairRows / kPairChunk;  // 16
constexpr int kPairMaxCpi = 16;                           // j-chunks per work item, at most
static_assert(kPairMaxCpi <= kPairBlockChunks && kPairBlockChunks % kPairMaxCpi == 0,
              "chunks per item must divide the chunks of an i-block");
}  // namespace gi
// Far-field sums of every body of the table's runs into a.fsum_fx (which
// must be zero on entry); then the epilogue, as gi_launch_finish.
cudaError_t gi_launch_pair_force(const ForceArgs &a, const LaunchTable &tab, cudaStream_t s);
cudaError_t gi_launch_pair_finish(int epi, const ForceArgs &a, const LaunchTable &tab, int maxn,
                                  int nsm, cudaStream_t s);

// gi_grid.cu: contact corrections of every body of the table's runs into
// delta (3 x int64 per body) through a hashed cell grid.  Its scratch layout
// is computed here, as constexpr functions, so that gi_noalloc.cu can check
// at compile time that its static array holds the largest run it accepts.
namespace gi {
// A bucket goes through the tiled path only when it holds at least this many
// bodies; that bounds the number of tiled buckets and work items.
constexpr unsigned int kDenseFloor = 32;
// Cost classes of the tiled path's work items (128-body tiles staged - 1).
constexpr unsigned int kItemClasses = 16;
// Tiled-path counters: items, tiled buckets, queue head, one spare, then a
// count and a fill cursor per cost class.
constexpr int kCtrWords = 4 + 2 * (int)kItemClasses;
}  // namespace gi

// Buckets of the grid for `bodies` bodies: a power of two >= 2 * bodies.
constexpr unsigned int gi_grid_buckets(long long bodies)
{
    unsigned long long m = 1024;
    while (m < 2ull * (unsigned long long)bodies) m <<= 1;
    return (unsigned int)m;
}

// Tiled-path work items: at most 27 per chunk of 128 bodies of a dense
// bucket, and a dense bucket holds at least kDenseFloor bodies, so at most
// 27 (bodies / 128 + bodies / kDenseFloor + 2).  Tiled buckets: each holds at
// least kDenseFloor bodies.
constexpr size_t gi_dense_item_capacity(long long bodies)
{
    return 27 * ((size_t)bodies / 128 + (size_t)bodies / gi::kDenseFloor + 2);
}
constexpr size_t gi_dense_bucket_capacity(long long bodies)
{
    return (size_t)bodies / gi::kDenseFloor + 1;
}

// Words of grid scratch: slot-ordered positions and velocities (float4, 8
// words per slot); keys (indexed by global body index) and sorted (by slot):
// max_end words each; cursor and bucket state: one word per bucket each;
// block sums: 8192; the tiled path's counters and up to 3 words to align the
// items to 16 bytes; items as listed and as ordered (4 words each); tiled
// buckets.
constexpr size_t gi_grid_words(long long max_end, long long bodies)
{
    return 8 * (size_t)bodies + 2 * (size_t)max_end + 2 * (size_t)gi_grid_buckets(bodies) + 8192 +
           gi::kCtrWords + 3 + 8 * gi_dense_item_capacity(bodies) +
           gi_dense_bucket_capacity(bodies);
}
// With s_warp and ev_grid given, the warp-per-body kernel runs on s_warp
// after the grid is built (ev_grid is recorded on s and waited on by
// s_warp); the caller then joins s_warp as well as s.
cudaError_t gi_launch_contacts(const float4 *pos, const float4 *vel, const LaunchTable &tab,
                               long long bodies, int max_end, unsigned int *work,
                               long long *delta, int nsm, cudaStream_t s,
                               cudaStream_t s_warp = nullptr, cudaEvent_t ev_grid = nullptr);

// gi_aux.cu
cudaError_t gi_launch_move(float4 *pos, float4 *vel, const float4 *force,
                           const LaunchTable &tab, cudaStream_t s);
// The diagnostics' blocks for pass 1 or 2: the resident blocks of that pass
// on sm_count SMs.
int gi_diag_blocks(int pass, int sm_count);
// Both passes of the FP64 diagnostics; work holds 16 doubles per block of
// the larger grid, out_dev 15 doubles, ticket 2 ints (cleared here).
cudaError_t gi_launch_diag(const float4 *pos, const float4 *vel,
                           const unsigned char *label, int scope,
                           const RunDev &run, float mass_fe, float mass_si, double *work,
                           int nblocks1, int nblocks2, double *out_dev, int *ticket,
                           cudaStream_t s);
cudaError_t gi_launch_potential(const float4 *pos, const LaunchTable &tab,
                                double *per_block, int nblocks_per_run,
                                cudaStream_t s);
cudaError_t gi_launch_ffma_peak(float *sink, int blocks, int iters, cudaStream_t s);

// gi_api.cu helpers for the library's other translation units: record an
// error for gi_last_error() and return `status`; the device pair table of a
// reference collision struct.
int gi_internal_fail(int status, const char *msg);
int gi_internal_collision_pairdev(const gi_force_collision_consts *c, PairDev *d);
// Device scratch bytes one run of n bodies needs in `ctx` (admission estimate).
long long gi_internal_scratch_bytes(gi_ctx *ctx, int n);
// The paired far field's decomposition of one run of n bodies with 2^pcl
// j-chunks per work item, its items numbered from item_start: fills the
// run's pcl ... far_inv and item_start, returns its work items.
long long gi_internal_pair_run(RunDev &d, int n, int pcl, const PairDev &p, long long item_start);
// log2 of the j-chunks per item of a run of n bodies without a tuning table.
int gi_internal_pair_default_pcl(int n);
// Device ordinal of a context (-1 for NULL).
int gi_internal_ctx_device(gi_ctx *ctx);
// Attempts one union-find link of gi_find_earth_moon may make (gi_options).
int gi_internal_ctx_cluster_tries(gi_ctx *ctx);
// gi_grid.cu: exclusive scan of m <= 1024 * 8192 counters in place; sums
// holds 8192 words of scratch.
cudaError_t gi_bucket_scan(unsigned int *a, unsigned int m, unsigned int *sums, cudaStream_t s);
