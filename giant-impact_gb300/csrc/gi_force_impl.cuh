// gi_force_impl.cuh -- the all-pairs force kernel (and its fused kick-drift
// epilogue) for sm_103a.  Included once per i-bodies-per-thread value by
// gi_force_ipt{1,2,4}.cu so those instances compile in parallel.
//
// Physics follows the reference pair law (Code/ImpactCode/impactAddTime.cu:
// 283-370): attraction G m_i m_j / r^2 for r >= 1, G m_i m_j - K (1 - r^2)
// inside one diameter, K chosen by the pair class and dropping to KR for a
// separating pair inside its shell.
//
// Work decomposition.  A work item is (run, i-block, j-chunk).  An i-block
// is GI_NT * IPT consecutive bodies of one run, one CTA of GI_NT threads,
// IPT bodies per thread (ILP).  j-chunks split the run's bodies so that
// small runs still fill all SMs; a chunk is processed in tiles of GI_NT
// bodies staged in shared memory and read back as broadcast LDS.128.
//
// r2 and dp.dv are formed as fma(z, z, fma(x, x, y*y)), the evaluation the
// reference's own build uses, so band and K/KR decisions see the identical
// FP32 r2 and dp.dv.
//
// Inner loop (per j, per i): 3 FADD, 1 FMUL + 2 FFMA (r2), MUFU.RSQ,
// 3 FMUL (m_j r^-3), compare + select, 3 FFMA: far-field gravity only.
// Pairs with r2 < 1 contribute zero there; when any lane of the warp has
// one, the warp runs the contact path for that j, which evaluates the full
// reference branch structure with IEEE sqrt / div (so its band and K/KR
// decisions are bit-identical to the reference) and the contact force
// G - K (1 - r^2) with 1 - r^2 carried exactly.
//
// Accumulation.  Each tile's sum is plain FP32 (128 terms); tiles are
// folded Kahan-compensated (GI_ACC_KAHAN), in FP64 (GI_ACC_FP64) or plainly
// (GI_ACC_FP32).  Split j-chunks leave FP64 partial sums in scratch; the
// last CTA of an i-block (atomic ticket) adds them in chunk order, so the
// result is deterministic and depends only on the run's decomposition.
#pragma once

#include "gi_internal.h"

namespace gi {

// MUFU reciprocal square root (PTX rsqrt.approx.ftz.f32).  Only pairs with
// r2 >= 1 use the value, so flushing denormal inputs changes nothing; r2 = 0
// (the self pair) gives +inf, which the contact mask discards.
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

// G - K (1 - r2) with 1 - r2 split exactly into dhi + dlo (Fast2Sum, valid
// because r2 < 1 here): one rounding when r2 >= 0.5 (dlo == 0), which is the
// float rounding of the reference's double expression.
__device__ __forceinline__ float contact_mag(float G, float K, float r2)
{
    float dhi = __fsub_rn(1.0f, r2);
    float dlo = __fsub_rn(__fsub_rn(1.0f, dhi), r2);
    return __fmaf_rn(-K, dlo, __fmaf_rn(-K, dhi, G));
}

// Contact-branch force of pair (i, j), accumulated into k{x,y,z}.
__device__ __forceinline__ void contact_pair(const PairDev &P, int sep_test,
                                             int i, int j, int sw, float dx,
                                             float dy, float dz, float r2,
                                             const float4 *__restrict__ vel,
                                             float4 vj, float &kx, float &ky,
                                             float &kz)
{
    const int test = (i < sw) + (j < sw);
    const float G = P.G[test];
    float K = P.K[test];
    if (!(r2 >= P.Tband[test])) {
        // Inside the shell: the separation test needs both velocities.
        const float4 vi = __ldg(&vel[i]);
        const float dvx = __fsub_rn(vj.x, vi.x), dvy = __fsub_rn(vj.y, vi.y),
                    dvz = __fsub_rn(vj.z, vi.z);
        const float dpdv = __fmaf_rn(dz, dvz, __fmaf_rn(dx, dvx, __fmul_rn(dy, dvy)));
        // Reference: int inout = dp.dv; KR when inout > 0, i.e. dp.dv >= 1.
        const bool sep = (sep_test == GI_SEP_SIGN) ? (dpdv > 0.0f) : (dpdv >= 1.0f);
        if (sep) K = (r2 >= P.Tmid[test]) ? P.KRmid[test] : P.KRin[test];
    }
    const float mag = contact_mag(G, K, r2);
    const float invr = (i == j) ? 0.0f : __fdiv_rn(1.0f, __fsqrt_rn(r2));
    kx = __fmaf_rn(__fmul_rn(mag, dx), invr, kx);
    ky = __fmaf_rn(__fmul_rn(mag, dy), invr, ky);
    kz = __fmaf_rn(__fmul_rn(mag, dz), invr, kz);
}

template <int IPT, int ACC, int EPI>
__global__ void __launch_bounds__(GI_NT)
force_kernel(const ForceArgs a, const __grid_constant__ LaunchTable tab)
{
    __shared__ float4 sP[GI_NT];
    __shared__ float4 sV[GI_NT];
    __shared__ int sLast;

    const int tid = threadIdx.x;
    const int item = blockIdx.x;
    const RunDev &R = tab.runs[find_run(tab, item)];
    const PairDev &P = tab.params[R.param];
    const int local = item - R.item_start;
    const int ib = local / R.nsplit;
    const int sp = local - ib * R.nsplit;
    const int rbeg = R.offset, rend = R.offset + R.n, sw = R.offset + R.nfe;
    const int i0 = rbeg + ib * (GI_NT * IPT);
    const int j0 = rbeg + sp * R.jchunk;
    const int j1 = min(j0 + R.jchunk, rend);
    const float4 *__restrict__ pos = a.pos;
    const float4 *__restrict__ vel = a.vel;

    float xi[IPT], yi[IPT], zi[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = i0 + k * GI_NT + tid;
        if (i < rend) {
            const float4 p = __ldg(&pos[i]);
            xi[k] = p.x; yi[k] = p.y; zi[k] = p.z;
        } else {
            xi[k] = GI_FAR_I; yi[k] = GI_FAR_I; zi[k] = GI_FAR_I;
        }
    }

    // Running sums: sum (+ compensation for Kahan, or double for FP64) and
    // the contact-force accumulators.
    float sx[IPT], sy[IPT], sz[IPT];
    float cx[IPT], cy[IPT], cz[IPT];
    double dxs[ACC == GI_ACC_FP64 ? IPT : 1], dys[ACC == GI_ACC_FP64 ? IPT : 1],
        dzs[ACC == GI_ACC_FP64 ? IPT : 1];
    float kx[IPT], ky[IPT], kz[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        sx[k] = sy[k] = sz[k] = 0.0f;
        cx[k] = cy[k] = cz[k] = 0.0f;
        kx[k] = ky[k] = kz[k] = 0.0f;
        if (ACC == GI_ACC_FP64) { dxs[k] = dys[k] = dzs[k] = 0.0; }
    }

    // Per-tile partial sums.  In GI_ACC_FP32 mode they are the running sums
    // themselves (plain sequential FP32 accumulation, no fold).
    float tx[IPT], ty[IPT], tz[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) tx[k] = ty[k] = tz[k] = 0.0f;

    for (int jt = j0; jt < j1; jt += GI_NT) {
        const int j = jt + tid;
        float4 pj, vj;
        if (j < j1) {
            pj = __ldg(&pos[j]);
            vj = __ldg(&vel[j]);
            pj.w = (j < sw) ? P.gm_fe : P.gm_si;
        } else {
            pj = make_float4(GI_FAR_J, GI_FAR_J, GI_FAR_J, 0.0f);
            vj = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        __syncthreads();
        sP[tid] = pj;
        sV[tid] = vj;
        __syncthreads();

        if (ACC != GI_ACC_FP32) {
#pragma unroll
            for (int k = 0; k < IPT; ++k) tx[k] = ty[k] = tz[k] = 0.0f;
        }

#pragma unroll 4
        for (int jj = 0; jj < GI_NT; ++jj) {
            const float4 q = sP[jj];
            bool anyc = false;
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const float dx = q.x - xi[k], dy = q.y - yi[k], dz = q.z - zi[k];
                const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
                const float ri = rsqrt_mufu(r2);
                float s = ri * ri;
                s = s * ri;
                s = s * q.w;
                const bool c = r2 < 1.0f;
                s = c ? 0.0f : s;
                anyc = anyc || c;
                tx[k] = __fmaf_rn(s, dx, tx[k]);
                ty[k] = __fmaf_rn(s, dy, ty[k]);
                tz[k] = __fmaf_rn(s, dz, tz[k]);
            }
            if (__any_sync(0xffffffffu, anyc)) {
                const float4 vq = sV[jj];
                const int jg = jt + jj;
#pragma unroll
                for (int k = 0; k < IPT; ++k) {
                    const int ig = i0 + k * GI_NT + tid;
                    const float dx = q.x - xi[k], dy = q.y - yi[k], dz = q.z - zi[k];
                    const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
                    // Padding never reaches here (it sits 1e16 away), but the
                    // contact path loads vel[i]: keep it inside the run regardless.
                    if (r2 < 1.0f && ig < rend && jg < j1)
                        contact_pair(P, tab.sep_test, ig, jg, sw, dx, dy, dz, r2, vel, vq,
                                     kx[k], ky[k], kz[k]);
                }
            }
        }

        // Fold this tile's partial sums.
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            if (ACC == GI_ACC_FP32) {
                // running sums stay in t
            } else if (ACC == GI_ACC_FP64) {
                dxs[k] += (double)tx[k]; dys[k] += (double)ty[k]; dzs[k] += (double)tz[k];
            } else {
                float y, t;
                y = tx[k] - cx[k]; t = sx[k] + y; cx[k] = (t - sx[k]) - y; sx[k] = t;
                y = ty[k] - cy[k]; t = sy[k] + y; cy[k] = (t - sy[k]) - y; sy[k] = t;
                y = tz[k] - cz[k]; t = sz[k] + y; cz[k] = (t - sz[k]) - y; sz[k] = t;
            }
        }
    }

    if (ACC == GI_ACC_FP32) {
#pragma unroll
        for (int k = 0; k < IPT; ++k) { sx[k] = tx[k]; sy[k] = ty[k]; sz[k] = tz[k]; }
    }

    // ---------------------------------------------------------------- epilogue
    // F = gm_i * A + C  (A = sum_j gm_j dp r^-3 over far pairs, C = contact).
    float fx[IPT], fy[IPT], fz[IPT];
    if (R.nsplit > 1) {
        const long long plane = (long long)R.n;
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = i0 + k * GI_NT + tid;
            if (i < rend) {
                const double gmi = (double)((i < sw) ? P.gm_fe : P.gm_si);
                double ax, ay, az;
                if (ACC == GI_ACC_FP64) { ax = dxs[k]; ay = dys[k]; az = dzs[k]; }
                else { ax = (double)sx[k] - (double)cx[k]; ay = (double)sy[k] - (double)cy[k]; az = (double)sz[k] - (double)cz[k]; }
                double *pp = a.partials + R.part_base + (long long)(sp * 3) * plane + (i - rbeg);
                pp[0] = gmi * ax + (double)kx[k];
                pp[plane] = gmi * ay + (double)ky[k];
                pp[2 * plane] = gmi * az + (double)kz[k];
            }
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            const unsigned int t = atomicAdd(&a.tickets[R.tick_base + ib], 1u);
            sLast = (t == (unsigned int)(R.nsplit - 1));
        }
        __syncthreads();
        if (!sLast) return;
        __threadfence();
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = i0 + k * GI_NT + tid;
            double ax = 0.0, ay = 0.0, az = 0.0;
            if (i < rend) {
                const double *pp = a.partials + R.part_base + (i - rbeg);
                for (int s2 = 0; s2 < R.nsplit; ++s2) {
                    const double *q = pp + (long long)(s2 * 3) * plane;
                    ax += __ldcg(q);
                    ay += __ldcg(q + plane);
                    az += __ldcg(q + 2 * plane);
                }
            }
            fx[k] = (float)ax; fy[k] = (float)ay; fz[k] = (float)az;
        }
        if (tid == 0) a.tickets[R.tick_base + ib] = 0u;
    } else {
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = i0 + k * GI_NT + tid;
            const float gmi = (i < sw) ? P.gm_fe : P.gm_si;
            if (ACC == GI_ACC_FP64) {
                fx[k] = (float)((double)gmi * dxs[k] + (double)kx[k]);
                fy[k] = (float)((double)gmi * dys[k] + (double)ky[k]);
                fz[k] = (float)((double)gmi * dzs[k] + (double)kz[k]);
            } else {
                fx[k] = __fmaf_rn(gmi, sx[k], __fmaf_rn(-gmi, cx[k], kx[k]));
                fy[k] = __fmaf_rn(gmi, sy[k], __fmaf_rn(-gmi, cy[k], ky[k]));
                fz[k] = __fmaf_rn(gmi, sz[k], __fmaf_rn(-gmi, cz[k], kz[k]));
            }
        }
    }

#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = i0 + k * GI_NT + tid;
        if (i >= rend) continue;
        if (EPI == GI_EPI_FORCE) {
            float *f = reinterpret_cast<float *>(a.force + i);
            f[0] = fx[k]; f[1] = fy[k]; f[2] = fz[k];
        } else {
            // v += (F - damp v) dt/m ; x += v dt  (impactAddTime.cu:384-393,
            // generateTargetImpactor.cu:636-663), .w carried through.
            const float dtm = (i < sw) ? R.dtm_fe : R.dtm_si;
            float4 v = __ldg(&vel[i]);
            float4 p = __ldg(&pos[i]);
            v.x = __fmaf_rn(__fmaf_rn(-R.damp, v.x, fx[k]), dtm, v.x);
            v.y = __fmaf_rn(__fmaf_rn(-R.damp, v.y, fy[k]), dtm, v.y);
            v.z = __fmaf_rn(__fmaf_rn(-R.damp, v.z, fz[k]), dtm, v.z);
            p.x = __fmaf_rn(v.x, R.dt, p.x);
            p.y = __fmaf_rn(v.y, R.dt, p.y);
            p.z = __fmaf_rn(v.z, R.dt, p.z);
            a.vel_out[i] = v;
            a.pos_out[i] = p;
        }
    }
}

template <int IPT>
cudaError_t launch_force_ipt(int acc, int epi, const ForceArgs &a,
                             const LaunchTable &tab, cudaStream_t s)
{
    if (tab.nitems <= 0) return cudaSuccess;
    dim3 grid(tab.nitems), block(GI_NT);
#define GI_CASE(A, E)                                                    \
    if (acc == A && epi == E) {                                          \
        force_kernel<IPT, A, E><<<grid, block, 0, s>>>(a, tab);          \
        return cudaGetLastError();                                       \
    }
    GI_CASE(GI_ACC_KAHAN, GI_EPI_FORCE)
    GI_CASE(GI_ACC_KAHAN, GI_EPI_STEP)
    GI_CASE(GI_ACC_FP32, GI_EPI_FORCE)
    GI_CASE(GI_ACC_FP32, GI_EPI_STEP)
    GI_CASE(GI_ACC_FP64, GI_EPI_FORCE)
    GI_CASE(GI_ACC_FP64, GI_EPI_STEP)
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
#undef GI_OCC
    return e == cudaSuccess ? nb : 0;
}

}  // namespace gi
