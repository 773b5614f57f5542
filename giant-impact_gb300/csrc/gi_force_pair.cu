// gi_force_pair.cu -- the far field with every unordered pair evaluated once
// (GI_ACCUM_PAIRED, the default accumulation mode).
//
// The law's far field is symmetric: the clamped gravity of a pair,
// G m_i m_j (x_j - x_i) / max(r, 1)^3, acts on i, and its negative on j
// (the pair law of Code/ImpactCode/impactAddTime.cu:283-370 for r >= 1,
// and the clamped term that gi_grid.cu corrects for r < 1).  The reference
// evaluates every ordered pair, each thread summing the force on its own
// body; here each pair is evaluated once and applied to both bodies, which
// cuts the pair arithmetic on the FMA pipe, the unit that bounds the far
// field, from 22 to about 15 lane operations per pair.
//
// Work decomposition.  An i-block is 1024 consecutive bodies of one run, one
// CTA of 4 warps, 8 bodies per lane held in registers (packed in pairs for
// FP32x2 arithmetic).  A j-chunk is 32 consecutive bodies of the run, one per
// lane.  A work item is (run, i-block a, a range of `cpi` chunks); block a
// takes the chunks from its own first body onwards, so every pair i < j is
// covered exactly once:
//   - a chunk wholly after a warp's 256 rows: every pair, unmasked;
//   - a chunk inside the warp's rows (the diagonal): only i < j;
//   - a chunk wholly before the warp's rows: skipped (the warp that owns
//     those bodies meets this warp's bodies as its j).
// Items are numbered block-major; block a has ceil((C - 32 a) / cpi) of them
// (C = chunks of the run; cpi divides 32, so this is k0 - a 32 / cpi and the
// items before block a are an arithmetic series, decoded by bisection).  CTA
// t of a run takes item (t * stride) mod items, the stride coprime with the
// item count and about one i-block's items long: CTAs resident together then
// hold different i-blocks, so their i-side atomics do not queue on the same
// addresses.
//
// Inner loop (per warp and chunk): the chunk is staged in shared memory as
// (x, y, z, gm).  Lane l starts with j = l; at step s it meets
// j = (l + s) mod 32 and adds the pair to its own 8 i-sums and to a running
// j-sum, which then moves one lane down (one shuffle per component).  After
// 32 steps the j-sum has visited every lane and is back on lane j, holding
// sum_i dp r^-3 over the warp's 256 i-bodies.  Per pair of i-bodies and
// step: 3 FADD2 (dp), FMUL2 + 2 FFMA2 (r2), 2 FMNMX, 2 MUFU.RSQ, 2 FMUL2
// (r^-3), 3 FFMA2 (i-sums), 3 FFMA2 (j-sum); per step 6 FADD fold the two
// halves of the j-sum.  14.75 FMA-pipe lane operations per pair.
//
// Masses (gm = sqrt(G) m, so G m_i m_j = gm_i gm_j).  The i-sums gather
// dp r^-3 over a chunk and are scaled by the chunk's gm_j when folded;
// chunks that straddle the Fe/Si boundary, and the diagonal ones, take the
// per-pair gm_j instead.  A warp's 256 rows are of one class except in the
// one warp per run that straddles the boundary: the others scale their
// finished i-sums and every j-sum by their gm_i, and only the straddling
// warp multiplies gm_i into each pair.  The j-sum is scaled by the lane's own
// gm_j and negated.
//
// Accumulation and determinism.  Chunk sums are FP32 (32 terms per i-body,
// 256 per j-body and warp); the i-sums of an item are added chunk by chunk
// in FP32 (at most 32 chunks).  Everything beyond that is 64-bit fixed point
// with a power-of-two unit chosen per run so that no sum of a body's pair
// terms can overflow it (|F| <= n gm_max^2 < 2^62 units): the j-sums of a CTA
// are added in shared memory, then both sides into one int64 triple per
// body in global memory.  Integer addition is associative, so the result
// does not depend on which CTA finished first: it depends only on the run's
// bodies, n and cpi.  pair_finish_kernel converts the sums, adds the contact
// corrections and stores the force or steps the bodies with the arithmetic
// of the one-sided kernel's epilogue.
#include <algorithm>

#include "gi_force_impl.cuh"

namespace gi {

constexpr int kPairH = kPairIpl / 2;  // packed pairs of i-bodies per lane

__device__ __forceinline__ long long pair_items_before(long long a, long long k0, long long q)
{
    return a * k0 - q * ((a * (a - 1)) / 2);
}

// One warp, one chunk.  cj: the chunk's 32 staged bodies (x, y, z, gm).
// di = (warp's first row) - (chunk's first body), relative to the run.
//   EDGE: a diagonal chunk (only i < j) or one that straddles the Fe/Si
//         boundary; the i-sums take the per-pair gm_j.
//   IMIX: the warp's rows straddle the Fe/Si boundary; w takes the per-row
//         gm_i.  Every other warp has one i mass, applied after the sums.
template <bool EDGE, bool IMIX>
__device__ __forceinline__ void pair_chunk(const float4 *__restrict__ cj, const int lane,
                                           const int di, const float2 (&nx)[kPairH],
                                           const float2 (&ny)[kPairH], const float2 (&nz)[kPairH],
                                           const float2 (&gi)[kPairH], float2 (&ax)[kPairH],
                                           float2 (&ay)[kPairH], float2 (&az)[kPairH],
                                           float &bx, float &by, float &bz)
{
    bx = by = bz = 0.0f;
#pragma unroll 4
    for (int s = 0; s < kPairChunk; ++s) {
        const int jl = (lane + s) & (kPairChunk - 1);
        const float4 q = cj[jl];
        const float2 X = make_float2(q.x, q.x), Y = make_float2(q.y, q.y),
                     Z = make_float2(q.z, q.z);
        float2 cx = make_float2(0.0f, 0.0f), cy = cx, cz = cx;
#pragma unroll
        for (int h = 0; h < kPairH; ++h) {
            const float2 dx = __fadd2_rn(X, nx[h]);
            const float2 dy = __fadd2_rn(Y, ny[h]);
            const float2 dz = __fadd2_rn(Z, nz[h]);
            // fma(dz, dz, fma(dx, dx, dy*dy)) per lane, as the reference
            float2 r2 = __fmul2_rn(dy, dy);
            r2 = __ffma2_rn(dx, dx, r2);
            r2 = __ffma2_rn(dz, dz, r2);
            const float2 ri = make_float2(rsqrt_mufu(fmaxf(r2.x, 1.0f)),
                                          rsqrt_mufu(fmaxf(r2.y, 1.0f)));
            float2 w = IMIX ? __fmul2_rn(__fmul2_rn(ri, ri), __fmul2_rn(ri, gi[h]))
                            : __fmul2_rn(__fmul2_rn(ri, ri), ri);
            float2 wi = w;
            if (EDGE) {
                // rows 2h and 2h+1 of this lane: i = di + (2h) 32 + lane
                const int i0 = di + 2 * h * 32 + lane;
                w.x = i0 < jl ? w.x : 0.0f;
                w.y = i0 + 32 < jl ? w.y : 0.0f;
                wi = __fmul2_rn(w, make_float2(q.w, q.w));
            }
            ax[h] = __ffma2_rn(wi, dx, ax[h]);
            ay[h] = __ffma2_rn(wi, dy, ay[h]);
            az[h] = __ffma2_rn(wi, dz, az[h]);
            cx = __ffma2_rn(w, dx, cx);
            cy = __ffma2_rn(w, dy, cy);
            cz = __ffma2_rn(w, dz, cz);
        }
        bx += cx.x + cx.y;
        by += cy.x + cy.y;
        bz += cz.x + cz.y;
        // the j-sum moves to the lane that meets this j next
        bx = __shfl_sync(0xffffffffu, bx, lane + 1);
        by = __shfl_sync(0xffffffffu, by, lane + 1);
        bz = __shfl_sync(0xffffffffu, bz, lane + 1);
    }
}

// One warp over the item's chunks.  The i-sums (sx, sy, sz) gather
// sum_chunks gm_j sum_j w dp; each chunk's j-sums go, times -gm_j and
// scale_j, into the CTA's fixed-point j-sums in shared memory.
template <bool IMIX>
__device__ __forceinline__ void pair_warp(const float4 *__restrict__ sp,
                                          unsigned long long *__restrict__ sj, const int c0,
                                          const int nch, const int wi0, const int lane,
                                          const int nfe, const PairDev &P, const float scale_j,
                                          const float2 (&nx)[kPairH], const float2 (&ny)[kPairH],
                                          const float2 (&nz)[kPairH], const float2 (&gi)[kPairH],
                                          float2 (&sx)[kPairH], float2 (&sy)[kPairH],
                                          float2 (&sz)[kPairH])
{
#pragma unroll 1
    for (int c = 0; c < nch; ++c) {
        const int jc0 = (c0 + c) * kPairChunk;  // relative to the run
        if (jc0 + kPairChunk <= wi0) continue;  // before this warp's rows
        const bool diag = jc0 < wi0 + kPairWarpRows;
        const bool straddle = jc0 < nfe && nfe < jc0 + kPairChunk;
        float2 ax[kPairH], ay[kPairH], az[kPairH];
#pragma unroll
        for (int h = 0; h < kPairH; ++h) ax[h] = ay[h] = az[h] = make_float2(0.0f, 0.0f);
        float bx, by, bz;
        float gc;  // the chunk's gm_j, applied at the fold (1 for EDGE chunks)
        if (diag || straddle) {
            pair_chunk<true, IMIX>(sp + c * kPairChunk, lane, wi0 - jc0, nx, ny, nz, gi, ax, ay,
                                   az, bx, by, bz);
            gc = 1.0f;
        } else {
            pair_chunk<false, IMIX>(sp + c * kPairChunk, lane, 0, nx, ny, nz, gi, ax, ay, az, bx,
                                    by, bz);
            gc = jc0 < nfe ? P.gm_fe : P.gm_si;
        }
        // j side: lane l holds j = jc0 + l; the force on j is -gm_j times its sum
        const float gj = -sp[c * kPairChunk + lane].w * scale_j;
        unsigned long long *dst = sj + (size_t)(c * kPairChunk + lane) * 3;
        atomicAdd(dst + 0, (unsigned long long)__float2ll_rn(gj * bx));
        atomicAdd(dst + 1, (unsigned long long)__float2ll_rn(gj * by));
        atomicAdd(dst + 2, (unsigned long long)__float2ll_rn(gj * bz));
        // i side: fold the chunk sum, scaled by the chunk's gm_j
        const float2 g2 = make_float2(gc, gc);
#pragma unroll
        for (int h = 0; h < kPairH; ++h) {
            sx[h] = __ffma2_rn(ax[h], g2, sx[h]);
            sy[h] = __ffma2_rn(ay[h], g2, sy[h]);
            sz[h] = __ffma2_rn(az[h], g2, sz[h]);
        }
    }
}

// 152 registers (no spills): 3 CTAs per SM use 58,368 of the 65,536, and a
// 64-thread block of the contact pass fits beside them on every SM (about
// 1 % per fused step against 168 registers, which fill the SM).
__global__ void __maxnreg__(152)
pair_force_kernel(const ForceArgs a, const __grid_constant__ LaunchTable tab)
{
    extern __shared__ float4 pair_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int item = blockIdx.x;
    const RunDev &R = tab.runs[find_run(tab, item)];
    const PairDev &P = tab.params[R.param];
    const int cpi = 1 << R.pcl;
    float4 *sp = pair_smem;                                       // cpi * 32 bodies
    unsigned long long *sj = reinterpret_cast<unsigned long long *>(pair_smem + cpi * kPairChunk);

    // ---- decode (i-block a, item k of the block).  Consecutive CTAs take
    // items a stride apart, so the CTAs running at once work on different
    // i-blocks and their sums land on different addresses.
    const long long t = ((long long)(item - R.item_start) * R.pstride) % R.pitems;
    const long long k0 = R.pk0, q = kPairBlockChunks >> R.pcl;
    int lo = 0, hi = R.pnb - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pair_items_before(mid, k0, q) <= t) lo = mid;
        else hi = mid - 1;
    }
    const int blk = lo;
    const int c0 = blk * kPairBlockChunks + (int)(t - pair_items_before(blk, k0, q)) * cpi;
    const int nch = min(cpi, R.pnc - c0);
    const int rbeg = R.offset, n = R.n, nfe = R.nfe;

    // ---- stage the j-range (x, y, z, gm_j), clear the j-sums
    for (int u = threadIdx.x; u < nch * kPairChunk; u += blockDim.x) {
        const int j = c0 * kPairChunk + u;  // relative to the run
        float4 v = make_float4(GI_FAR_J, GI_FAR_J, GI_FAR_J, 0.0f);
        if (j < n) {
            const float4 p = __ldg(&a.pos[rbeg + j]);
            v = make_float4(p.x, p.y, p.z, j < nfe ? P.gm_fe : P.gm_si);
        }
        sp[u] = v;
    }
    for (int u = threadIdx.x; u < nch * kPairChunk * 3; u += blockDim.x) sj[u] = 0ull;

    // ---- this lane's 8 i-bodies: rows wi0 + k 32 + lane, k = 0..7.  Rows
    // beyond the run sit at GI_FAR_I, where r^-3 underflows to zero.
    const int wi0 = blk * kPairRows + warp * kPairWarpRows;  // relative to the run
    float2 nx[kPairH], ny[kPairH], nz[kPairH], gi[kPairH];
#pragma unroll
    for (int h = 0; h < kPairH; ++h) {
        float4 p2[2];
        float g2[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int i = wi0 + (2 * h + e) * 32 + lane;
            p2[e] = make_float4(GI_FAR_I, GI_FAR_I, GI_FAR_I, 0.0f);
            g2[e] = 0.0f;
            if (i < n) {
                p2[e] = __ldg(&a.pos[rbeg + i]);
                g2[e] = i < nfe ? P.gm_fe : P.gm_si;
            }
        }
        nx[h] = make_float2(-p2[0].x, -p2[1].x);
        ny[h] = make_float2(-p2[0].y, -p2[1].y);
        nz[h] = make_float2(-p2[0].z, -p2[1].z);
        gi[h] = make_float2(g2[0], g2[1]);
    }
    float2 sx[kPairH], sy[kPairH], sz[kPairH];
#pragma unroll
    for (int h = 0; h < kPairH; ++h) sx[h] = sy[h] = sz[h] = make_float2(0.0f, 0.0f);
    // A warp whose rows are all of one class takes its gm_i out of the pair
    // loop: it scales the j-sums and the finished i-sums instead.
    const bool imix = wi0 < nfe && nfe < wi0 + kPairWarpRows;
    const float gmw = imix ? 1.0f : (wi0 < nfe ? P.gm_fe : P.gm_si);
    const float inv = R.far_inv, scale_i = inv * gmw;
    __syncthreads();

    if (imix)
        pair_warp<true>(sp, sj, c0, nch, wi0, lane, nfe, P, inv, nx, ny, nz, gi, sx, sy, sz);
    else
        pair_warp<false>(sp, sj, c0, nch, wi0, lane, nfe, P, scale_i, nx, ny, nz, gi, sx, sy,
                         sz);

    // ---- i side into the global fixed-point sums
    unsigned long long *out = reinterpret_cast<unsigned long long *>(a.fsum_fx);
#pragma unroll
    for (int h = 0; h < kPairH; ++h) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int i = wi0 + (2 * h + e) * 32 + lane;
            if (i >= n) continue;
            unsigned long long *o = out + 3 * (size_t)(rbeg + i);
            const float vx = e ? sx[h].y : sx[h].x, vy = e ? sy[h].y : sy[h].x,
                        vz = e ? sz[h].y : sz[h].x;
            atomicAdd(o + 0, (unsigned long long)__float2ll_rn(vx * scale_i));
            atomicAdd(o + 1, (unsigned long long)__float2ll_rn(vy * scale_i));
            atomicAdd(o + 2, (unsigned long long)__float2ll_rn(vz * scale_i));
        }
    }
    // ---- j side of the whole CTA
    __syncthreads();
    unsigned long long *oj = out + 3 * ((size_t)rbeg + (size_t)c0 * kPairChunk);
    const int nj = min(nch * kPairChunk, n - c0 * kPairChunk);
    for (int u = threadIdx.x; u < nj * 3; u += blockDim.x) {
        const unsigned long long v = sj[u];
        if (v) atomicAdd(oj + u, v);
    }
}

// The epilogue: F = fixed-point far field + contact correction, rounded once
// to float, stored (GI_EPI_FORCE) or applied as the kick-drift (GI_EPI_STEP)
// by finish_body, the one-sided kernel's own epilogue arithmetic.
template <int EPI>
__global__ void __launch_bounds__(256) pair_finish_kernel(const ForceArgs a,
                                                          const __grid_constant__ LaunchTable tab)
{
    const RunDev &R = tab.runs[blockIdx.y];
    const double unit = tab.params[R.param].fx_unit;
    const double far_unit = R.far_unit;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < R.n; k += gridDim.x * blockDim.x) {
        const int i = R.offset + k;
        const long long *q = a.fsum_fx + 3 * (size_t)i;
        const double fd[3] = {(double)__ldcg(q) * far_unit, (double)__ldcg(q + 1) * far_unit,
                              (double)__ldcg(q + 2) * far_unit};
        finish_body<EPI>(a, R, unit, i, fd);
    }
}

}  // namespace gi

using namespace gi;

cudaError_t gi_launch_pair_force(const ForceArgs &a, const LaunchTable &tab, cudaStream_t s)
{
    if (tab.nitems <= 0) return cudaSuccess;
    int pcl = 0;
    for (int r = 0; r < tab.nruns; ++r) pcl = std::max(pcl, tab.runs[r].pcl);
    const size_t smem = (size_t)(1 << pcl) * kPairChunk * (sizeof(float4) + 3 * sizeof(long long));
    pair_force_kernel<<<tab.nitems, kPairWarps * 32, smem, s>>>(a, tab);
    return cudaGetLastError();
}

cudaError_t gi_launch_pair_finish(int epi, const ForceArgs &a, const LaunchTable &tab, int maxn,
                                  int nsm, cudaStream_t s)
{
    if (tab.nruns <= 0 || maxn <= 0) return cudaSuccess;
    const int bx = std::max(1, std::min((maxn + 255) / 256, 4 * nsm));
    dim3 grid(bx, tab.nruns);
    if (epi == GI_EPI_FORCE) pair_finish_kernel<GI_EPI_FORCE><<<grid, 256, 0, s>>>(a, tab);
    else if (epi == GI_EPI_STEP) pair_finish_kernel<GI_EPI_STEP><<<grid, 256, 0, s>>>(a, tab);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}
