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
// field, from 22 to 14 lane operations per pair.
//
// Work decomposition.  An i-block is 1024 consecutive bodies of one run, one
// CTA of 4 warps, 8 bodies per lane held in registers.  A j-chunk is 64
// consecutive bodies of the run, two per lane (slots l and l + 32).  A work
// item is (run, i-block a, a range of `cpi` chunks); block a takes the
// chunks from its own first body onwards, so every pair i < j is covered
// exactly once:
//   - a chunk wholly after a warp's 256 rows: every pair, unmasked;
//   - a chunk inside the warp's rows (the diagonal): only i < j;
//   - a chunk wholly before the warp's rows: skipped (the warp that owns
//     those bodies meets this warp's bodies as its j).
// Items are numbered block-major; block a has ceil((C - 16 a) / cpi) of them
// (C = chunks of the run; cpi divides 16, so this is k0 - a 16 / cpi and the
// items before block a are an arithmetic series, decoded by bisection).  CTA
// t of a run takes item (t * stride) mod items, the stride coprime with the
// item count and about one i-block's items long: CTAs resident together then
// hold different i-blocks, so their i-side atomics do not queue on the same
// addresses.
//
// Inner loop (per warp and chunk): the chunk is staged in shared memory as
// (x_a, x_b, y_a, y_b) and (z_a, z_b, gm_a, gm_b) of slots a = l, b = l + 32,
// so one lane's two j-bodies fill the two halves of an FP32x2 register; each
// i-body is held duplicated in both halves.  Lane l starts with slots
// (l, l + 32); at step s it meets slots ((l + s) mod 32, + 32) and adds the
// 16 pairs to its 8 i-sums (one half per j) and to the two j-sums, which
// then move one lane down (one shuffle per half and component).  After 32
// steps the j-sums have visited every lane and are back on their lanes.  Per
// i-body and step, all packed: 3 FADD2 (dp), FMUL2 + 2 FFMA2 (r2), 2 FMNMX,
// 2 MUFU.RSQ, 2 FMUL2 (r^-3), 3 FFMA2 (i-sums), 3 FFMA2 (j-sums): 14
// FMA-pipe lane operations per pair, with no per-step fold of the j-sums
// (each half is one j's).
//
// Masses (gm = sqrt(G) m, so G m_i m_j = gm_i gm_j).  The i-sums gather
// dp r^-3 over a chunk and are scaled by the chunk's gm_j when folded;
// chunks that straddle the Fe/Si boundary, and the diagonal ones, take the
// per-pair gm_j instead.  A warp's 256 rows are of one class except in the
// one warp per run that straddles the boundary: the others scale their
// finished i-sums and every j-sum by their gm_i, and only the straddling
// warp multiplies gm_i into each pair.  The j-sums are scaled by their own
// gm_j and negated.
//
// Accumulation and determinism.  Chunk sums are FP32 (32 terms a half per
// i-body, 256 a half per j-body and warp); a chunk's two halves are folded
// into the i-body's running FP32 sum in shared memory (at most 16 chunks an
// item).  Everything beyond that is 64-bit fixed point with a power-of-two
// unit chosen per run so that no sum of a body's pair terms can overflow it
// (|F| <= n gm_max^2 < 2^62 units): the j-sums of a CTA are added in shared
// memory, then both sides into one int64 triple per body in global memory.
// Integer addition is associative, so the result does not depend on which
// CTA finished first: it depends only on the run's bodies, n and cpi.
// pair_finish_kernel converts the sums, adds the contact corrections and
// stores the force or steps the bodies with the arithmetic of the one-sided
// kernel's epilogue.
#include <algorithm>
#include <atomic>

#include "gi_force_impl.cuh"

namespace gi {

__device__ __forceinline__ long long pair_items_before(long long a, long long k0, long long q)
{
    return a * k0 - q * ((a * (a - 1)) / 2);
}

// One warp, one 64-body chunk, two j-bodies a lane.  cxy[l] = (x_a, x_b,
// y_a, y_b) and czg[l] = (z_a, z_b, gm_a, gm_b) of chunk slots a = l and
// b = l + 32.  di = (warp's first row) - (chunk's first body), relative to
// the run.
//   EDGE: a diagonal chunk (only i < j) or one that straddles the Fe/Si
//         boundary; the i-sums take the per-pair gm_j.
//   IMIX: the warp's rows straddle the Fe/Si boundary; w takes the per-row
//         gm_i.  Every other warp has one i mass, applied after the sums.
// ax[k] (per component) gathers row k's terms, one half per j of the lane.
template <bool EDGE, bool IMIX>
__device__ __forceinline__ void pair_chunk(const float4 *__restrict__ cxy,
                                           const float4 *__restrict__ czg, const int lane,
                                           const int di, const float2 (&nx)[kPairIpl],
                                           const float2 (&ny)[kPairIpl],
                                           const float2 (&nz)[kPairIpl],
                                           const float2 (&gi)[kPairIpl], float2 (&ax)[kPairIpl],
                                           float2 (&ay)[kPairIpl], float2 (&az)[kPairIpl],
                                           float2 &bx, float2 &by, float2 &bz)
{
    bx = by = bz = make_float2(0.0f, 0.0f);
#pragma unroll 2
    for (int s = 0; s < 32; ++s) {
        const int jl = (lane + s) & 31;
        const float4 q = cxy[jl];
        const float4 g = czg[jl];
        const float2 X = make_float2(q.x, q.y), Y = make_float2(q.z, q.w),
                     Z = make_float2(g.x, g.y);
#pragma unroll
        for (int k = 0; k < kPairIpl; ++k) {
            const float2 dx = __fadd2_rn(X, nx[k]);
            const float2 dy = __fadd2_rn(Y, ny[k]);
            const float2 dz = __fadd2_rn(Z, nz[k]);
            // fma(dz, dz, fma(dx, dx, dy*dy)) per lane, as the reference
            float2 r2 = __fmul2_rn(dy, dy);
            r2 = __ffma2_rn(dx, dx, r2);
            r2 = __ffma2_rn(dz, dz, r2);
            const float2 ri = make_float2(rsqrt_mufu(fmaxf(r2.x, 1.0f)),
                                          rsqrt_mufu(fmaxf(r2.y, 1.0f)));
            float2 w = IMIX ? __fmul2_rn(__fmul2_rn(ri, ri), __fmul2_rn(ri, gi[k]))
                            : __fmul2_rn(__fmul2_rn(ri, ri), ri);
            float2 wi = w;
            if (EDGE) {
                const int i = di + k * 32 + lane;  // this row, relative to the chunk
                w.x = i < jl ? w.x : 0.0f;
                w.y = i < jl + 32 ? w.y : 0.0f;
                wi = __fmul2_rn(w, make_float2(g.z, g.w));
            }
            ax[k] = __ffma2_rn(wi, dx, ax[k]);
            ay[k] = __ffma2_rn(wi, dy, ay[k]);
            az[k] = __ffma2_rn(wi, dz, az[k]);
            bx = __ffma2_rn(w, dx, bx);
            by = __ffma2_rn(w, dy, by);
            bz = __ffma2_rn(w, dz, bz);
        }
        // the j-sums move to the lane that meets these j next
        bx.x = __shfl_sync(0xffffffffu, bx.x, lane + 1);
        bx.y = __shfl_sync(0xffffffffu, bx.y, lane + 1);
        by.x = __shfl_sync(0xffffffffu, by.x, lane + 1);
        by.y = __shfl_sync(0xffffffffu, by.y, lane + 1);
        bz.x = __shfl_sync(0xffffffffu, bz.x, lane + 1);
        bz.y = __shfl_sync(0xffffffffu, bz.y, lane + 1);
    }
}

// One warp over the item's chunks.  Row r's running i-sum (si[d * 1024 + r],
// shared memory) gathers sum_chunks gm_j sum_j w dp; each chunk's j-sums go,
// times -gm_j and scale_j, into the CTA's fixed-point j-sums.
template <bool IMIX>
__device__ __forceinline__ void pair_warp(const float4 *__restrict__ cxy,
                                          const float4 *__restrict__ czg,
                                          unsigned long long *__restrict__ sj,
                                          float *__restrict__ si, const int c0, const int nch,
                                          const int wi0, const int warp, const int lane,
                                          const int nfe, const PairDev &P, const float scale_j,
                                          const float2 (&nx)[kPairIpl],
                                          const float2 (&ny)[kPairIpl],
                                          const float2 (&nz)[kPairIpl],
                                          const float2 (&gi)[kPairIpl])
{
#pragma unroll 1
    for (int c = 0; c < nch; ++c) {
        const int jc0 = (c0 + c) * kPairChunk;  // relative to the run
        if (jc0 + kPairChunk <= wi0) continue;  // before this warp's rows
        const bool diag = jc0 < wi0 + kPairWarpRows;
        const bool straddle = jc0 < nfe && nfe < jc0 + kPairChunk;
        float2 ax[kPairIpl], ay[kPairIpl], az[kPairIpl];
#pragma unroll
        for (int k = 0; k < kPairIpl; ++k) ax[k] = ay[k] = az[k] = make_float2(0.0f, 0.0f);
        float2 bx, by, bz;
        float gc;  // the chunk's gm_j, applied at the fold (1 for EDGE chunks)
        if (diag || straddle) {
            pair_chunk<true, IMIX>(cxy + c * 32, czg + c * 32, lane, wi0 - jc0, nx, ny, nz, gi,
                                   ax, ay, az, bx, by, bz);
            gc = 1.0f;
        } else {
            pair_chunk<false, IMIX>(cxy + c * 32, czg + c * 32, lane, 0, nx, ny, nz, gi, ax, ay,
                                    az, bx, by, bz);
            gc = jc0 < nfe ? P.gm_fe : P.gm_si;
        }
        // j side: lane l holds j = jc0 + l (.x) and jc0 + 32 + l (.y); the
        // force on j is -gm_j times its sum
        const float4 g = czg[c * 32 + lane];
        const float ga = -g.z * scale_j, gb = -g.w * scale_j;
        unsigned long long *da = sj + (size_t)(c * kPairChunk + lane) * 3;
        unsigned long long *db = sj + (size_t)(c * kPairChunk + 32 + lane) * 3;
        atomicAdd(da + 0, (unsigned long long)__float2ll_rn(ga * bx.x));
        atomicAdd(da + 1, (unsigned long long)__float2ll_rn(ga * by.x));
        atomicAdd(da + 2, (unsigned long long)__float2ll_rn(ga * bz.x));
        atomicAdd(db + 0, (unsigned long long)__float2ll_rn(gb * bx.y));
        atomicAdd(db + 1, (unsigned long long)__float2ll_rn(gb * by.y));
        atomicAdd(db + 2, (unsigned long long)__float2ll_rn(gb * bz.y));
        // i side: the two halves, scaled by the chunk's gm_j, into the
        // running sums (each thread owns its rows: no atomics)
#pragma unroll
        for (int k = 0; k < kPairIpl; ++k) {
            const int r = warp * kPairWarpRows + k * 32 + lane;
            si[r] = __fmaf_rn(ax[k].x + ax[k].y, gc, si[r]);
            si[kPairRows + r] = __fmaf_rn(ay[k].x + ay[k].y, gc, si[kPairRows + r]);
            si[2 * kPairRows + r] = __fmaf_rn(az[k].x + az[k].y, gc, si[2 * kPairRows + r]);
        }
    }
}

// Shared memory of one work item of 2^pcl chunks.
__host__ __device__ constexpr size_t pair_smem_bytes(int pcl)
{
    return (size_t)(1 << pcl) * 32 * (2 * sizeof(float4)) +
           (size_t)(1 << pcl) * kPairChunk * 3 * sizeof(unsigned long long) +
           3 * (size_t)kPairRows * sizeof(float);
}

// 152 registers (no spills): 3 CTAs per SM use 58,368 of the 65,536, and a
// 64-thread block of the contact pass fits beside them on every SM.
__global__ void __maxnreg__(152)
pair_force_kernel(const ForceArgs a, const __grid_constant__ LaunchTable tab)
{
    extern __shared__ float4 pair_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int item = blockIdx.x;
    const RunDev &R = tab.runs[find_run(tab, item)];
    const PairDev &P = tab.params[R.param];
    const int cpi = 1 << R.pcl;
    float4 *cxy = pair_smem;                  // cpi * 32: (x_a, x_b, y_a, y_b)
    float4 *czg = pair_smem + cpi * 32;       // cpi * 32: (z_a, z_b, gm_a, gm_b)
    unsigned long long *sj =
        reinterpret_cast<unsigned long long *>(pair_smem + 2 * cpi * 32);  // cpi * 64 * 3
    float *si = reinterpret_cast<float *>(sj + (size_t)cpi * kPairChunk * 3);  // 3 * 1024

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

    // ---- stage the j-range, clear the j-sums and the running i-sums
    for (int u = threadIdx.x; u < nch * 32; u += blockDim.x) {
        const int ja = (c0 + (u >> 5)) * kPairChunk + (u & 31), jb = ja + 32;  // relative to the run
        float4 pa = make_float4(GI_FAR_J, GI_FAR_J, GI_FAR_J, 0.0f), pb = pa;
        float ga = 0.0f, gb = 0.0f;
        if (ja < n) {
            pa = __ldg(&a.pos[rbeg + ja]);
            ga = ja < nfe ? P.gm_fe : P.gm_si;
        }
        if (jb < n) {
            pb = __ldg(&a.pos[rbeg + jb]);
            gb = jb < nfe ? P.gm_fe : P.gm_si;
        }
        cxy[u] = make_float4(pa.x, pb.x, pa.y, pb.y);
        czg[u] = make_float4(pa.z, pb.z, ga, gb);
    }
    for (int u = threadIdx.x; u < nch * kPairChunk * 3; u += blockDim.x) sj[u] = 0ull;
    for (int u = threadIdx.x; u < 3 * kPairRows; u += blockDim.x) si[u] = 0.0f;

    // ---- this lane's 8 i-bodies: rows wi0 + k 32 + lane, k = 0..7, each
    // duplicated in both halves of its registers.  Rows beyond the run sit
    // at GI_FAR_I, where r^-3 underflows to zero.
    const int wi0 = blk * kPairRows + warp * kPairWarpRows;  // relative to the run
    float2 nx[kPairIpl], ny[kPairIpl], nz[kPairIpl], gi[kPairIpl];
#pragma unroll
    for (int k = 0; k < kPairIpl; ++k) {
        const int i = wi0 + k * 32 + lane;
        float4 p = make_float4(GI_FAR_I, GI_FAR_I, GI_FAR_I, 0.0f);
        float g = 0.0f;
        if (i < n) {
            p = __ldg(&a.pos[rbeg + i]);
            g = i < nfe ? P.gm_fe : P.gm_si;
        }
        nx[k] = make_float2(-p.x, -p.x);
        ny[k] = make_float2(-p.y, -p.y);
        nz[k] = make_float2(-p.z, -p.z);
        gi[k] = make_float2(g, g);
    }
    // A warp whose rows are all of one class takes its gm_i out of the pair
    // loop: it scales the j-sums and the finished i-sums instead.
    const bool imix = wi0 < nfe && nfe < wi0 + kPairWarpRows;
    const float gmw = imix ? 1.0f : (wi0 < nfe ? P.gm_fe : P.gm_si);
    const float inv = R.far_inv, scale_i = inv * gmw;
    __syncthreads();

    if (imix)
        pair_warp<true>(cxy, czg, sj, si, c0, nch, wi0, warp, lane, nfe, P, inv, nx, ny, nz, gi);
    else
        pair_warp<false>(cxy, czg, sj, si, c0, nch, wi0, warp, lane, nfe, P, scale_i, nx, ny, nz,
                         gi);

    // ---- i side into the global fixed-point sums
    unsigned long long *out = reinterpret_cast<unsigned long long *>(a.fsum_fx);
#pragma unroll
    for (int k = 0; k < kPairIpl; ++k) {
        const int i = wi0 + k * 32 + lane;
        if (i >= n) continue;
        const int r = warp * kPairWarpRows + k * 32 + lane;
        unsigned long long *o = out + 3 * (size_t)(rbeg + i);
        atomicAdd(o + 0, (unsigned long long)__float2ll_rn(si[r] * scale_i));
        atomicAdd(o + 1, (unsigned long long)__float2ll_rn(si[kPairRows + r] * scale_i));
        atomicAdd(o + 2, (unsigned long long)__float2ll_rn(si[2 * kPairRows + r] * scale_i));
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
    const size_t smem = pair_smem_bytes(pcl);
    // Items of more than 8 chunks take more than the 48 KB of shared memory
    // a kernel gets by default: raise its limit once per device (the first
    // such launch on a device comes before any capture, which cannot grow
    // scratch either).
    static std::atomic<int> raised[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (smem > (48u << 10) && dev >= 0 && dev < 64 && !raised[dev].load()) {
        e = cudaFuncSetAttribute(pair_force_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)pair_smem_bytes(4));
        if (e != cudaSuccess) return e;
        raised[dev].store(1);
    }
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
