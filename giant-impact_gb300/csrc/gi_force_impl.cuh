// gi_force_impl.cuh -- the all-pairs force kernel (and its fused kick-drift
// epilogue) for sm_103a.  Included once per i-bodies-per-thread value by
// gi_force_ipt{1,2,4,8}.cu so those instances compile in parallel.
//
// Physics follows the reference pair law (Code/ImpactCode/impactAddTime.cu:
// 283-370): attraction G m_i m_j / r^2 for r >= 1, G m_i m_j - K (1 - r^2)
// inside one diameter, K chosen by the pair class and dropping to KR for a
// separating pair inside its shell.  The work is split in two:
//   - this kernel: gravity of every pair with r^2 clamped at one diameter,
//     G m_i m_j dp / max(r, 1)^3, branch-free, the O(N^2) part;
//   - gi_grid.cu: for the pairs with r^2 < 1 (found through a cell grid) the
//     reference's contact force minus the clamped term added here, summed in
//     64-bit fixed point; the epilogue below adds it.
// r2 is formed as fma(z, z, fma(x, x, y*y)), the evaluation of the
// reference's own build, in both places.
//
// Work decomposition.  A work item is (run, i-block, j-chunk).  An i-block
// is GI_NT * IPT consecutive bodies of one run, handled by one CTA of GI_NT
// threads, IPT bodies per thread (ILP).  j-chunks split the run's bodies so
// that small runs still fill all SMs: chunks of 2^lg tiles of GI_NT bodies,
// the last lg of them shrinking 2^(lg-1), ..., 2, 1 tiles.  A chunk is walked
// in tiles of GI_NT positions staged in shared memory and read back as
// broadcast LDS.128.  The kernel is persistent: one resident wave of CTAs
// pulls items (largest first) from an atomic queue.
//
// Inner loop: two j-bodies at a time in packed FP32x2 instructions (sm_100+
// FADD2 / FMUL2 / FFMA2), per i-body and j pair: 3 FADD2, FMUL2 + 2 FFMA2
// (r2), 2 FMNMX (clamp), 2 MUFU.RSQ, 2 FMUL2 (r^-3), 3 FFMA2 -- 15 issue
// slots for two interactions.  j-tiles never straddle the Fe/Si boundary,
// so the j mass is applied once per tile, not per pair.
//
// Accumulation.  Each tile's sum is plain FP32 (at most 128 terms); tiles
// are folded Kahan-compensated (GI_ACC_KAHAN), in FP64 (GI_ACC_FP64) or
// plainly (GI_ACC_FP32).  Split j-chunks leave FP64 partial sums in scratch;
// the last CTA of an i-block (atomic ticket) adds them in chunk order, so
// the result is deterministic and depends only on the run's decomposition.
#pragma once

#include "gi_internal.h"

namespace gi {

// MUFU reciprocal square root (PTX rsqrt.approx.ftz.f32).  Only inputs >= 1
// reach it (r2 is clamped), so flushing denormals changes nothing.
__device__ __forceinline__ float rsqrt_mufu(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ int find_run(const LaunchTable &tab, int item)
{
    int lo = 0, hi = tab.nruns - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tab.runs[mid].item_start <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Tiles covered by the last r chunks of a run.  Counted from the end the
// chunks have 1, 2, 4, ..., 2^lg tiles, then 2^lg tiles each (the first
// chunk of the run takes what is left), so the queue, which hands out
// chunk 0 of every i-block first, ends on the smallest items.
__device__ __forceinline__ int tail_tiles(int r, int lg)
{
    return (r <= lg) ? (1 << r) - 1 : (1 << lg) - 1 + (r - lg) * (1 << lg);
}

// G - K (1 - r2) with 1 - r2 split exactly into dhi + dlo (Fast2Sum, valid
// because r2 < 1 here): one rounding when r2 >= 0.5 (dlo == 0), which is the
// float rounding of the reference's double expression.
__device__ __forceinline__ float contact_mag(float G, float K, float r2)
{
    float dhi = __fsub_rn(1.0f, r2);
    float dlo = __fsub_rn(__fsub_rn(1.0f, dhi), r2);
    return __fmaf_rn(-K, dlo, __fmaf_rn(-K, dhi, G));
}

// F = far-field sum + contact correction, rounded once to float; stored as
// the force (GI_EPI_FORCE) or applied as the kick-drift into the other
// state buffer (GI_EPI_STEP).  Shared by the fused epilogue and
// finish_kernel, so both give the same bits.
template <int EPI>
__device__ __forceinline__ void finish_body(const ForceArgs &a, const RunDev &R, double unit,
                                            int i, const double fd[3])
{
    const long long *dl = a.delta + 3 * (size_t)i;
    const float fx = (float)(fd[0] + (double)__ldcg(dl + 0) * unit);
    const float fy = (float)(fd[1] + (double)__ldcg(dl + 1) * unit);
    const float fz = (float)(fd[2] + (double)__ldcg(dl + 2) * unit);
    if (EPI == GI_EPI_FORCE) {
        float *f = reinterpret_cast<float *>(a.force + i);
        f[0] = fx; f[1] = fy; f[2] = fz;
    } else {
        // v += (F - damp v) dt/m ; x += v dt  (impactAddTime.cu:384-393,
        // generateTargetImpactor.cu:636-663), .w carried through.
        const float dtm = (i < R.offset + R.nfe) ? R.dtm_fe : R.dtm_si;
        float4 v = __ldg(&a.vel[i]);
        float4 p = __ldg(&a.pos[i]);
        v.x = __fmaf_rn(__fmaf_rn(-R.damp, v.x, fx), dtm, v.x);
        v.y = __fmaf_rn(__fmaf_rn(-R.damp, v.y, fy), dtm, v.y);
        v.z = __fmaf_rn(__fmaf_rn(-R.damp, v.z, fz), dtm, v.z);
        p.x = __fmaf_rn(v.x, R.dt, p.x);
        p.y = __fmaf_rn(v.y, R.dt, p.y);
        p.z = __fmaf_rn(v.z, R.dt, p.z);
        a.vel_out[i] = v;
        a.pos_out[i] = p;
    }
}

// Shared memory of one CTA: the staged j-tile and the running sums of its
// GI_NT * IPT i-bodies.  The sums are touched once per tile (the fold), so
// they live here rather than in registers.
template <int IPT, int ACC>
struct ForceSmem {
    // j-tile as pairs of bodies: A[p] = (x_2p, x_2p+1, y_2p, y_2p+1),
    // B[p] = (z_2p, z_2p+1), read with one LDS.128 + one LDS.64 per pair.
    float4 A[GI_NT / 2];
    float2 B[GI_NT / 2];
    float s[ACC == GI_ACC_FP64 ? 1 : IPT][3][GI_NT];   // running sum
    float c[ACC == GI_ACC_KAHAN ? IPT : 1][3][GI_NT];  // Kahan compensation
    double d[ACC == GI_ACC_FP64 ? IPT : 1][3][GI_NT];  // FP64 running sum
    int item;
    int last;
};

template <int IPT, int ACC, int EPI>
__device__ __forceinline__ void process_item(const int item, const ForceArgs &a,
                                             const LaunchTable &tab, ForceSmem<IPT, ACC> &sm)
{
    const int tid = threadIdx.x;
    const RunDev &R = tab.runs[find_run(tab, item)];
    const PairDev &P = tab.params[R.param];
    // Items are numbered chunk-major (every i-block's chunk 0, then chunk 1,
    // ...), and chunks shrink from big to a halving tail down to one tile,
    // so the queue ends on small items and the CTAs finish together.
    const int local = item - R.item_start;
    const int sp = local / R.nib;
    const int ib = local - sp * R.nib;
    const int rbeg = R.offset, rend = R.offset + R.n, sw = R.offset + R.nfe;
    const int i0 = rbeg + ib * (GI_NT * IPT);
    int j0 = rbeg, j1 = rend;
    if (R.nsplit > 1) {
        const int r = R.nsplit - 1 - sp;  // chunk index counted from the end
        j0 = rbeg + GI_NT * max(0, R.tiles - tail_tiles(r + 1, R.lg));
        j1 = min(rbeg + GI_NT * (R.tiles - tail_tiles(r, R.lg)), rend);
    }
    const float4 *__restrict__ pos = a.pos;

    // -x_i in both halves of a pair register: dp of two j at once is one FADD2.
    float2 nx[IPT], ny[IPT], nz[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = i0 + k * GI_NT + tid;
        float4 p = make_float4(GI_FAR_I, GI_FAR_I, GI_FAR_I, 0.0f);
        if (i < rend) p = __ldg(&pos[i]);
        nx[k] = make_float2(-p.x, -p.x);
        ny[k] = make_float2(-p.y, -p.y);
        nz[k] = make_float2(-p.z, -p.z);
        // A = sum_j gm_j dp max(r, 1)^-3
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (ACC == GI_ACC_FP64) sm.d[k][d][tid] = 0.0;
            else sm.s[k][d][tid] = 0.0f;
            if (ACC == GI_ACC_KAHAN) sm.c[k][d][tid] = 0.0f;
        }
    }

    // The chunk is walked in two segments, Fe j-bodies then Si j-bodies, so
    // every tile has one j mass: the inner loop sums dp r^-3 and the mass is
    // applied once per tile when the tile sum is folded.
#pragma unroll 1
    for (int seg = 0; seg < 2; ++seg) {
        const int s0 = seg == 0 ? j0 : max(j0, sw);
        const int s1 = seg == 0 ? min(j1, sw) : j1;
        const float gseg = seg == 0 ? P.gm_fe : P.gm_si;
#pragma unroll 1
        for (int jt = s0; jt < s1; jt += GI_NT) {
            const int j = jt + tid;
            const float4 pj = (j < s1) ? __ldg(&pos[j])
                                       : make_float4(GI_FAR_J, GI_FAR_J, GI_FAR_J, 0.0f);
            __syncthreads();
            {
                float *a = reinterpret_cast<float *>(&sm.A[tid >> 1]);
                float *b = reinterpret_cast<float *>(&sm.B[tid >> 1]);
                a[tid & 1] = pj.x;
                a[2 + (tid & 1)] = pj.y;
                b[tid & 1] = pj.z;
            }
            __syncthreads();

            // Two partial sums per component (even and odd j of the tile).
            float2 tx[IPT], ty[IPT], tz[IPT];
#pragma unroll
            for (int k = 0; k < IPT; ++k)
                tx[k] = ty[k] = tz[k] = make_float2(0.0f, 0.0f);

#pragma unroll(IPT >= 8 ? 2 : (IPT >= 4 ? 4 : 32))
            for (int jp = 0; jp < GI_NT / 2; ++jp) {
                const float4 qa = sm.A[jp];
                const float2 qz = sm.B[jp];
                const float2 qx = make_float2(qa.x, qa.y), qy = make_float2(qa.z, qa.w);
#pragma unroll
                for (int k = 0; k < IPT; ++k) {
                    const float2 dx = __fadd2_rn(qx, nx[k]);
                    const float2 dy = __fadd2_rn(qy, ny[k]);
                    const float2 dz = __fadd2_rn(qz, nz[k]);
                    // fma(dz, dz, fma(dx, dx, dy*dy)) per lane, as the reference
                    float2 r2 = __fmul2_rn(dy, dy);
                    r2 = __ffma2_rn(dx, dx, r2);
                    r2 = __ffma2_rn(dz, dz, r2);
                    // Clamped at one diameter: contact pairs (and the self
                    // pair, dp = 0) add a bounded term the contact pass removes.
                    const float2 ri = make_float2(rsqrt_mufu(fmaxf(r2.x, 1.0f)),
                                                  rsqrt_mufu(fmaxf(r2.y, 1.0f)));
                    const float2 sc = __fmul2_rn(__fmul2_rn(ri, ri), ri);
                    tx[k] = __ffma2_rn(sc, dx, tx[k]);
                    ty[k] = __ffma2_rn(sc, dy, ty[k]);
                    tz[k] = __ffma2_rn(sc, dz, tz[k]);
                }
            }

            // Fold this tile (times its j mass) into the running sums.
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const float t3[3] = {tx[k].x + tx[k].y, ty[k].x + ty[k].y, tz[k].x + tz[k].y};
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if (ACC == GI_ACC_FP32) {
                        sm.s[k][d][tid] += gseg * t3[d];
                    } else if (ACC == GI_ACC_FP64) {
                        sm.d[k][d][tid] += (double)gseg * (double)t3[d];
                    } else {
                        const float s0v = sm.s[k][d][tid];
                        const float y = gseg * t3[d] - sm.c[k][d][tid];
                        const float t = s0v + y;
                        sm.c[k][d][tid] = (t - s0v) - y;
                        sm.s[k][d][tid] = t;
                    }
                }
            }
        }
    }

    // ---------------------------------------------------------------- epilogue
    // F = gm_i A + contact correction, rounded once to float.
    const double unit = P.fx_unit;
    double fd[IPT][3];
    if (R.nsplit > 1) {
        const long long plane = (long long)R.n;
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = i0 + k * GI_NT + tid;
            if (i < rend) {
                const double gmi = (double)((i < sw) ? P.gm_fe : P.gm_si);
                double *pp = a.partials + R.part_base + (long long)(sp * 3) * plane + (i - rbeg);
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    double ax;
                    if (ACC == GI_ACC_FP64) ax = sm.d[k][d][tid];
                    else if (ACC == GI_ACC_KAHAN)
                        ax = (double)sm.s[k][d][tid] - (double)sm.c[k][d][tid];
                    else ax = (double)sm.s[k][d][tid];
                    pp[d * plane] = gmi * ax;
                }
            }
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            const unsigned int t = atomicAdd(&a.tickets[R.tick_base + ib], 1u);
            sm.last = (t == (unsigned int)(R.nsplit - 1));
        }
        __syncthreads();
        if (!sm.last) return;
        __threadfence();
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = i0 + k * GI_NT + tid;
            fd[k][0] = fd[k][1] = fd[k][2] = 0.0;
            if (i < rend) {
                const double *pp = a.partials + R.part_base + (i - rbeg);
                for (int s2 = 0; s2 < R.nsplit; ++s2) {
                    const double *q = pp + (long long)(s2 * 3) * plane;
                    fd[k][0] += __ldcg(q);
                    fd[k][1] += __ldcg(q + plane);
                    fd[k][2] += __ldcg(q + 2 * plane);
                }
            }
        }
        if (tid == 0) a.tickets[R.tick_base + ib] = 0u;
    } else {
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = i0 + k * GI_NT + tid;
            const double gmi = (double)((i < sw) ? P.gm_fe : P.gm_si);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                double ax;
                if (ACC == GI_ACC_FP64) ax = sm.d[k][d][tid];
                else if (ACC == GI_ACC_KAHAN)
                    ax = (double)sm.s[k][d][tid] - (double)sm.c[k][d][tid];
                else ax = (double)sm.s[k][d][tid];
                fd[k][d] = gmi * ax;
            }
        }
    }

#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = i0 + k * GI_NT + tid;
        if (i >= rend) continue;
        if (EPI == GI_EPI_SUM) {  // finish_kernel adds the contacts once they are done
            double *q = a.fsum + 3 * (size_t)i;
            q[0] = fd[k][0];
            q[1] = fd[k][1];
            q[2] = fd[k][2];
        } else {
            finish_body<EPI>(a, R, unit, i, fd[k]);
        }
    }
}

// Persistent kernel: gridDim.x resident CTAs pull work items from an atomic
// queue (a.queue[0]) until the table is exhausted.  The last CTA to leave
// (a.queue[1] counts departures) resets both counters for the next launch
// on the stream.  No CTA ever waits on another.
template <int IPT, int ACC, int EPI>
__global__ void __launch_bounds__(GI_NT)
force_kernel(const ForceArgs a, const __grid_constant__ LaunchTable tab)
{
    __shared__ ForceSmem<IPT, ACC> sm;
    for (;;) {
        __syncthreads();  // every thread has read sm.item of the last round
        if (threadIdx.x == 0) sm.item = (int)atomicAdd(&a.queue[0], 1u);
        __syncthreads();
        const int item = sm.item;
        if (item >= tab.nitems) break;
        process_item<IPT, ACC, EPI>(item, a, tab, sm);
    }
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int d = atomicAdd(&a.queue[1], 1u);
        if (d == gridDim.x - 1) {
            a.queue[0] = 0u;
            a.queue[1] = 0u;
        }
    }
}

template <int IPT>
cudaError_t launch_force_ipt(int acc, int epi, const ForceArgs &a, const LaunchTable &tab,
                             int grid, cudaStream_t s)
{
    if (tab.nitems <= 0) return cudaSuccess;
    if (grid < 1 || grid > tab.nitems) grid = tab.nitems;
    dim3 g(grid), block(GI_NT);
#define GI_CASE(A, E)                                                    \
    if (acc == A && epi == E) {                                          \
        force_kernel<IPT, A, E><<<g, block, 0, s>>>(a, tab);             \
        return cudaGetLastError();                                       \
    }
    GI_CASE(GI_ACC_KAHAN, GI_EPI_FORCE)
    GI_CASE(GI_ACC_KAHAN, GI_EPI_STEP)
    GI_CASE(GI_ACC_FP32, GI_EPI_FORCE)
    GI_CASE(GI_ACC_FP32, GI_EPI_STEP)
    GI_CASE(GI_ACC_FP64, GI_EPI_FORCE)
    GI_CASE(GI_ACC_FP64, GI_EPI_STEP)
    GI_CASE(GI_ACC_KAHAN, GI_EPI_SUM)
    GI_CASE(GI_ACC_FP32, GI_EPI_SUM)
    GI_CASE(GI_ACC_FP64, GI_EPI_SUM)
#undef GI_CASE
    return cudaErrorInvalidValue;
}

template <int IPT>
int occupancy_ipt(int acc, int epi)
{
    int nb = 0;
    cudaError_t e = cudaErrorInvalidValue;
#define GI_OCC(A, E)                                                              \
    if (acc == A && epi == E)                                                     \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, force_kernel<IPT, A, E>, GI_NT, 0);
    GI_OCC(GI_ACC_KAHAN, GI_EPI_FORCE)
    GI_OCC(GI_ACC_KAHAN, GI_EPI_STEP)
    GI_OCC(GI_ACC_FP32, GI_EPI_FORCE)
    GI_OCC(GI_ACC_FP32, GI_EPI_STEP)
    GI_OCC(GI_ACC_FP64, GI_EPI_FORCE)
    GI_OCC(GI_ACC_FP64, GI_EPI_STEP)
    GI_OCC(GI_ACC_KAHAN, GI_EPI_SUM)
    GI_OCC(GI_ACC_FP32, GI_EPI_SUM)
    GI_OCC(GI_ACC_FP64, GI_EPI_SUM)
#undef GI_OCC
    return e == cudaSuccess ? nb : 0;
}

// The far field's epilogue, split off (GI_EPI_SUM): one thread per body of
// the run blockIdx.y adds the contact corrections to the FP64 sums in fsum
// and stores the force or applies the kick-drift, as the fused epilogue does.
template <int EPI>
__global__ void __launch_bounds__(256) finish_kernel(const ForceArgs a,
                                                     const __grid_constant__ LaunchTable tab)
{
    const RunDev &R = tab.runs[blockIdx.y];
    const double unit = tab.params[R.param].fx_unit;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < R.n; k += gridDim.x * blockDim.x) {
        const int i = R.offset + k;
        const double *q = a.fsum + 3 * (size_t)i;
        const double fd[3] = {__ldcg(q), __ldcg(q + 1), __ldcg(q + 2)};
        finish_body<EPI>(a, R, unit, i, fd);
    }
}

}  // namespace gi
