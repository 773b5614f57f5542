// gi_aux.cu -- the memory-bound kernels around the force pass: kick-drift,
// FP64 diagnostic reductions, the pair potential, and the FFMA throughput
// microbenchmark that gives the force kernel its roofline denominator.
#include "gi_internal.h"

namespace gi {

// v += (F - damp v) dt/m ; x += v dt, w carried through.
// Reference: moveBodiesCollisionSingleGPU (Code/ImpactCode/impactAddTime.cu:
// 379-394) and moveBodiesDampedSeperate (Code/GenerateTargetImpactorCode/
// generateTargetImpactor.cu:628-664).  80 B per body (read pos, vel, force;
// write pos, vel).
__global__ void __launch_bounds__(256)
move_kernel(float4 *__restrict__ pos, float4 *__restrict__ vel,
            const float4 *__restrict__ force, const __grid_constant__ LaunchTable tab)
{
    const RunDev &R = tab.runs[blockIdx.y];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= R.n) return;
    const int i = R.offset + k;
    const float dtm = (k < R.nfe) ? R.dtm_fe : R.dtm_si;
    const float4 f = __ldg(&force[i]);
    float4 v = vel[i];
    float4 p = pos[i];
    v.x = __fmaf_rn(__fmaf_rn(-R.damp, v.x, f.x), dtm, v.x);
    v.y = __fmaf_rn(__fmaf_rn(-R.damp, v.y, f.y), dtm, v.y);
    v.z = __fmaf_rn(__fmaf_rn(-R.damp, v.z, f.z), dtm, v.z);
    p.x = __fmaf_rn(v.x, R.dt, p.x);
    p.y = __fmaf_rn(v.y, R.dt, p.y);
    p.z = __fmaf_rn(v.z, R.dt, p.z);
    vel[i] = v;
    pos[i] = p;
}

// ----------------------------------------------------------------- diag --

__device__ __forceinline__ bool in_scope(const unsigned char *label, int i, int scope)
{
    if (label == nullptr || scope == 0) return true;
    const unsigned char l = label[i];
    if (scope == 1) return l == 1 || l == 2;
    if (scope == 2) return l == 1;
    if (scope == 3) return l == 2;
    return l == 3;
}

// The sums of the diagnostics are kept per thread in float-float pairs on
// the FP32 pipe: a value is hi + lo, about 48 significant bits.  TwoSum and
// the FMA form of TwoProd are error-free, and every addition renormalises
// the pair, so a thread's sum of n terms is exact to about n 2^-48 of the
// terms' magnitudes.  This GPU issues FP64 at a small fraction of its FP32
// rate: with the per-body work in FP64 the two passes ran at ~850 GB/s, with
// it on the FP32 pipe they are bound by HBM.  FP64 remains for the block
// partials and everything after them.
struct FF {
    float hi, lo;
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// a += xh + xl, renormalised (|lo| <= ulp(hi) / 2).
__device__ __forceinline__ void ff_add2(FF &a, float xh, float xl)
{
    float s, e;
    two_sum(a.hi, xh, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, xl));
    a.hi = __fadd_rn(s, e);
    a.lo = __fsub_rn(e, __fsub_rn(a.hi, s));
}

__device__ __forceinline__ void ff_add(FF &a, float x) { ff_add2(a, x, 0.0f); }

// a += x * y, the product taken exactly (p + e with e = fma(x, y, -p)).
__device__ __forceinline__ void ff_add_prod(FF &a, float x, float y)
{
    const float p = __fmul_rn(x, y);
    ff_add2(a, p, __fmaf_rn(x, y, -p));
}

// x - c for a float x and a double c given as ch + cl (ch = (float)c):
// TwoSum of x and -ch is exact, cl is folded into the low part.
__device__ __forceinline__ FF ff_sub_d(float x, float ch, float cl)
{
    FF r;
    float e;
    two_sum(x, -ch, r.hi, e);
    r.lo = __fsub_rn(e, cl);
    return r;
}

// a += u v - w z for float-float u, v, w, z: each product's high part
// exact, its cross terms to 2^-24 of themselves, the lo * lo terms
// (2^-48 of the product) left out.
__device__ __forceinline__ void ff_add_cross(FF &a, FF u, FF v, FF w, FF z)
{
    const float p1 = __fmul_rn(u.hi, v.hi);
    float e1 = __fmaf_rn(u.hi, v.hi, -p1);
    e1 = __fmaf_rn(u.hi, v.lo, __fmaf_rn(u.lo, v.hi, e1));
    const float p2 = __fmul_rn(w.hi, z.hi);
    float e2 = __fmaf_rn(w.hi, z.hi, -p2);
    e2 = __fmaf_rn(w.hi, z.lo, __fmaf_rn(w.lo, z.hi, e2));
    float s, t;
    two_sum(p1, -p2, s, t);
    ff_add2(a, s, __fadd_rn(t, __fsub_rn(e1, e2)));
}

__device__ __forceinline__ double ff_value(const FF &a) { return (double)a.hi + (double)a.lo; }

// Sum of the lanes' pairs to lane 0 (float-float), NV of them.
template <int NV>
__device__ __forceinline__ void warp_ff_sum(FF (&v)[NV])
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            const float h = __shfl_down_sync(0xffffffffu, v[c].hi, o);
            const float l = __shfl_down_sync(0xffffffffu, v[c].lo, o);
            ff_add2(v[c], h, l);
        }
    }
}

// Lane 0 of each warp passes its values (FP64); the block's warps are
// added in warp order and thread c < NV writes value c of the block.
template <int NV>
__device__ __forceinline__ void block_store(const double (&v)[NV], double *dst)
{
    __shared__ double sh[NV][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < NV; ++c) sh[c][warp] = v[c];
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double x = 0.0;
        const int nw = blockDim.x >> 5;
        for (int w = 0; w < nw; ++w) x += sh[threadIdx.x][w];
        dst[threadIdx.x] = x;
    }
}

// Both passes give each block one material class, so the class mass
// multiplies the block's sums once, in FP64: blocks [0, nbfe) take the
// run's Fe bodies [0, nfe), blocks [nbfe, gridDim.x) its Si bodies [nfe, n),
// each class in a grid-stride loop over its own blocks (nbfe in proportion
// to nfe).  Block b's partials are work[16 b ..].
__device__ __forceinline__ void class_range(int nfe, int n, int nbfe, double mfe, double msi,
                                            int &k0, int &k1, int &b, int &nb, double &m)
{
    const bool fe = (int)blockIdx.x < nbfe;
    k0 = fe ? 0 : nfe;
    k1 = fe ? nfe : n;
    b = fe ? (int)blockIdx.x : (int)blockIdx.x - nbfe;
    nb = fe ? nbfe : (int)gridDim.x - nbfe;
    m = fe ? mfe : msi;
}

// Pass 1: mass, sum m x, sum m v, kinetic energy, count (9 doubles / block).
__global__ void __launch_bounds__(256)
diag_pass1(const float4 *__restrict__ pos, const float4 *__restrict__ vel,
           const unsigned char *__restrict__ label, int scope, int off, int n,
           int nfe, int nbfe, double mfe, double msi, double *__restrict__ work)
{
    int k0, k1, b, nb;
    double m;
    class_range(nfe, n, nbfe, mfe, msi, k0, k1, b, nb, m);
    FF v[7];
#pragma unroll
    for (int c = 0; c < 7; ++c) v[c] = FF{0.0f, 0.0f};
    int cnt = 0;
    const auto body = [&](float4 p, float4 u) {
        ff_add(v[0], p.x);
        ff_add(v[1], p.y);
        ff_add(v[2], p.z);
        ff_add(v[3], u.x);
        ff_add(v[4], u.y);
        ff_add(v[5], u.z);
        ff_add_prod(v[6], u.x, u.x);
        ff_add_prod(v[6], u.y, u.y);
        ff_add_prod(v[6], u.z, u.z);
        ++cnt;
    };
    // two bodies' loads in flight at a time; each thread still takes its
    // bodies in grid-stride order
    const int stride = nb * blockDim.x;
    int k = k0 + b * blockDim.x + threadIdx.x;
    for (; k + stride < k1; k += 2 * stride) {
        const int i0 = off + k, i1 = i0 + stride;
        const float4 p0 = pos[i0], u0 = vel[i0], p1 = pos[i1], u1 = vel[i1];
        if (in_scope(label, i0, scope)) body(p0, u0);
        if (in_scope(label, i1, scope)) body(p1, u1);
    }
    if (k < k1 && in_scope(label, off + k, scope)) body(pos[off + k], vel[off + k]);
    warp_ff_sum<7>(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    const double d[9] = {m * cnt,
                         m * ff_value(v[0]), m * ff_value(v[1]), m * ff_value(v[2]),
                         m * ff_value(v[3]), m * ff_value(v[4]), m * ff_value(v[5]),
                         0.5 * m * ff_value(v[6]), (double)cnt};
    block_store<9>(d, work + 16 * blockIdx.x);
}

// Block partials summed in a fixed order (thread t takes blocks t, t + 256,
// ..., then a tree over the threads): deterministic.  Run as one block of
// 256 threads; the sums end in sh[c][0].
template <int NV>
__device__ __forceinline__ void ordered_sums(const double *__restrict__ work, int nblocks,
                                             double (&sh)[NV][256])
{
    const int t = threadIdx.x;
    double v[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) v[c] = 0.0;
    for (int b = t; b < nblocks; b += 256)
#pragma unroll
        for (int c = 0; c < NV; ++c) v[c] += work[16 * b + c];
#pragma unroll
    for (int c = 0; c < NV; ++c) sh[c][t] = v[c];
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (t < s)
#pragma unroll
            for (int c = 0; c < NV; ++c) sh[c][t] += sh[c][t + s];
        __syncthreads();
    }
}

// Finalise pass 1; out = [mass, com3, vcom3, -, -, -, ke, p3, count].
__global__ void __launch_bounds__(256) diag_fin1(const double *__restrict__ work, int nblocks,
                                                 double *out)
{
    __shared__ double sh[9][256];
    ordered_sums<9>(work, nblocks, sh);
    if (threadIdx.x != 0) return;
    const double m = sh[0][0];
    out[0] = m;
    for (int c = 0; c < 3; ++c) {
        out[1 + c] = m > 0.0 ? sh[1 + c][0] / m : 0.0;
        out[4 + c] = m > 0.0 ? sh[4 + c][0] / m : 0.0;
        out[11 + c] = sh[4 + c][0];
    }
    out[10] = sh[7][0];
    out[14] = sh[8][0];
}

// Pass 2: angular momentum about the com, relative to the com velocity
// (impactBasicFunctions.h:507-652 in double): r = x - com and w = v - vcom
// as float-float pairs, sum of r x w per class.
__global__ void __launch_bounds__(256)
diag_pass2(const float4 *__restrict__ pos, const float4 *__restrict__ vel,
           const unsigned char *__restrict__ label, int scope, int off, int n,
           int nfe, int nbfe, double mfe, double msi, const double *__restrict__ out,
           double *__restrict__ work)
{
    int k0, k1, b, nb;
    double m;
    class_range(nfe, n, nbfe, mfe, msi, k0, k1, b, nb, m);
    float ch[6], cl[6];  // com xyz, vcom xyz as float pairs
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const double x = out[1 + c];
        ch[c] = (float)x;
        cl[c] = (float)(x - (double)ch[c]);
    }
    FF L[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) L[c] = FF{0.0f, 0.0f};
    const auto body = [&](float4 p, float4 u) {
        const FF rx = ff_sub_d(p.x, ch[0], cl[0]), ry = ff_sub_d(p.y, ch[1], cl[1]),
                 rz = ff_sub_d(p.z, ch[2], cl[2]);
        const FF wx = ff_sub_d(u.x, ch[3], cl[3]), wy = ff_sub_d(u.y, ch[4], cl[4]),
                 wz = ff_sub_d(u.z, ch[5], cl[5]);
        ff_add_cross(L[0], ry, wz, rz, wy);
        ff_add_cross(L[1], rz, wx, rx, wz);
        ff_add_cross(L[2], rx, wy, ry, wx);
    };
    const int stride = nb * blockDim.x;
    int k = k0 + b * blockDim.x + threadIdx.x;
    for (; k + stride < k1; k += 2 * stride) {
        const int i0 = off + k, i1 = i0 + stride;
        const float4 p0 = pos[i0], u0 = vel[i0], p1 = pos[i1], u1 = vel[i1];
        if (in_scope(label, i0, scope)) body(p0, u0);
        if (in_scope(label, i1, scope)) body(p1, u1);
    }
    if (k < k1 && in_scope(label, off + k, scope)) body(pos[off + k], vel[off + k]);
    warp_ff_sum<3>(L);
    const double d[3] = {m * ff_value(L[0]), m * ff_value(L[1]), m * ff_value(L[2])};
    block_store<3>(d, work + 16 * blockIdx.x);
}

__global__ void __launch_bounds__(256) diag_fin2(const double *__restrict__ work, int nblocks,
                                                 double *out)
{
    __shared__ double sh[3][256];
    ordered_sums<3>(work, nblocks, sh);
    if (threadIdx.x != 0) return;
    out[7] = sh[0][0]; out[8] = sh[1][0]; out[9] = sh[2][0];
}

// -------------------------------------------------------------- potential --
// Per i-block of 128 bodies, sum over every j of the run of U(r_ij):
// far pairs -gm_i gm_j / r (FP32, rsqrt refined by one Newton step), contact
// pairs the full-K polynomial; 128-term tiles folded in FP64.  One double
// per block (already halved), summed by the host in block order.
__global__ void __launch_bounds__(GI_NT)
potential_kernel(const float4 *__restrict__ pos, const __grid_constant__ LaunchTable tab,
                 double *__restrict__ per_block)
{
    __shared__ float4 sP[GI_NT];
    __shared__ double sRed[GI_NT / 32];
    const int tid = threadIdx.x;
    // Locate the run: runs[r].item_start is the first block of run r.
    int lo = 0, hi = tab.nruns - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tab.runs[mid].item_start <= (int)blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    const RunDev &R = tab.runs[lo];
    const PairDev &P = tab.params[R.param];
    const int rbeg = R.offset, rend = R.offset + R.n, sw = R.offset + R.nfe;
    const int i = rbeg + (blockIdx.x - R.item_start) * GI_NT + tid;
    const bool valid = i < rend;
    float xi = GI_FAR_I, yi = GI_FAR_I, zi = GI_FAR_I;
    if (valid) { const float4 p = pos[i]; xi = p.x; yi = p.y; zi = p.z; }
    const bool ife = i < sw;
    double acc = 0.0;
    for (int jt = rbeg; jt < rend; jt += GI_NT) {
        const int j = jt + tid;
        float4 pj;
        if (j < rend) { pj = pos[j]; pj.w = (j < sw) ? P.gm_fe : P.gm_si; }
        else pj = make_float4(GI_FAR_J, GI_FAR_J, GI_FAR_J, 0.0f);
        __syncthreads();
        sP[tid] = pj;
        __syncthreads();
        float far = 0.0f, near = 0.0f;
#pragma unroll 4
        for (int jj = 0; jj < GI_NT; ++jj) {
            const float4 q = sP[jj];
            const float dx = q.x - xi, dy = q.y - yi, dz = q.z - zi;
            const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
            const bool c = r2 < 1.0f;
            // Contact pairs (and the self pair, r2 == 0) are taken out of the
            // far sum; rr keeps rsqrt finite for them.
            const float rr = c ? 1.0f : r2;
            float ri = rsqrtf(rr);
            ri = ri * __fmaf_rn(-0.5f * rr, ri * ri, 1.5f);  // one Newton-Raphson step
            far = __fmaf_rn(c ? 0.0f : q.w, ri, far);
            if (c && (jt + jj) != i && valid) {
                const int test = ife + ((jt + jj) < sw);
                const float G = P.G[test], K = P.K[test];
                const float r = __fsqrt_rn(r2);
                const float u = -G + G * (r - 1.0f) - K * (r - r * r * r * (1.0f / 3.0f) - 2.0f / 3.0f);
                near += u;
            }
        }
        const float gmi = ife ? P.gm_fe : P.gm_si;
        acc += -(double)gmi * (double)far + (double)near;
    }
    if (!valid) acc = 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((tid & 31) == 0) sRed[tid >> 5] = acc;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < GI_NT / 32; ++w) t += sRed[w];
        per_block[blockIdx.x] = 0.5 * t;
    }
}

// ------------------------------------------------------------ FFMA peak --
// Eight independent FMA chains per thread; 2 flops per FMA.
__global__ void __launch_bounds__(256) ffma_peak_kernel(float *sink, int iters)
{
    float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
    float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
    const float m = 0.9999999f, c = 1e-7f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = __fmaf_rn(a0, m, c); a1 = __fmaf_rn(a1, m, c);
            a2 = __fmaf_rn(a2, m, c); a3 = __fmaf_rn(a3, m, c);
            a4 = __fmaf_rn(a4, m, c); a5 = __fmaf_rn(a5, m, c);
            a6 = __fmaf_rn(a6, m, c); a7 = __fmaf_rn(a7, m, c);
        }
    }
    const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 1234.5f) sink[blockIdx.x] = s;
}

}  // namespace gi

cudaError_t gi_launch_move(float4 *pos, float4 *vel, const float4 *force,
                           const LaunchTable &tab, cudaStream_t s)
{
    int maxn = 0;
    for (int r = 0; r < tab.nruns; ++r) maxn = tab.runs[r].n > maxn ? tab.runs[r].n : maxn;
    if (maxn == 0 || tab.nruns == 0) return cudaSuccess;
    dim3 grid((maxn + 255) / 256, tab.nruns), block(256);
    gi::move_kernel<<<grid, block, 0, s>>>(pos, vel, force, tab);
    return cudaGetLastError();
}

cudaError_t gi_launch_diag(const float4 *pos, const float4 *vel,
                           const unsigned char *label, int scope,
                           const RunDev &run, const PairDev &par, float mass_fe,
                           float mass_si, double *work, int nblocks, double *out_dev,
                           cudaStream_t s)
{
    (void)par;
    // blocks for the Fe bodies in proportion to their number (at least one
    // when there are any), the rest for the Si bodies
    if (nblocks < 2) return cudaErrorInvalidValue;
    int nbfe = run.n > 0 ? (int)((long long)nblocks * run.nfe / run.n) : 0;
    if (run.nfe > 0 && nbfe < 1) nbfe = 1;
    if (nbfe > nblocks - 1) nbfe = nblocks - 1;
    gi::diag_pass1<<<nblocks, 256, 0, s>>>(pos, vel, label, scope, run.offset, run.n, run.nfe,
                                           nbfe, mass_fe, mass_si, work);
    gi::diag_fin1<<<1, 256, 0, s>>>(work, nblocks, out_dev);
    gi::diag_pass2<<<nblocks, 256, 0, s>>>(pos, vel, label, scope, run.offset, run.n, run.nfe,
                                           nbfe, mass_fe, mass_si, out_dev, work);
    gi::diag_fin2<<<1, 256, 0, s>>>(work, nblocks, out_dev);
    return cudaGetLastError();
}

cudaError_t gi_launch_potential(const float4 *pos, const LaunchTable &tab,
                                double *per_block, int nblocks, cudaStream_t s)
{
    if (nblocks <= 0) return cudaSuccess;
    gi::potential_kernel<<<nblocks, GI_NT, 0, s>>>(pos, tab, per_block);
    return cudaGetLastError();
}

cudaError_t gi_launch_ffma_peak(float *sink, int blocks, int iters, cudaStream_t s)
{
    gi::ffma_peak_kernel<<<blocks, 256, 0, s>>>(sink, iters);
    return cudaGetLastError();
}
