// gi_grid.cu -- contact forces through a hashed cell grid.
//
// The all-pairs kernel evaluates far-field gravity for every pair with r2
// clamped at one diameter.  The pairs inside one diameter (r2 < 1, the only
// ones where the reference law departs from gravity) are handled here:
//
//   1. grid: every body gets the cell floor(x), floor(y), floor(z) (cell size
//      D = 1, so two bodies within r < 1 are in the same or adjacent cells),
//      hashed with its run into M = 2^k buckets; a counting sort (histogram,
//      exclusive scan, scatter) lists the bodies of each bucket and copies
//      their state into slot order.
//   2. contact law: for each j of the same run with FP32 r2 < 1, the pass
//      adds the contact force of the reference law minus the clamped
//      far-field term the all-pairs pass added for that pair.  Band and K/KR
//      choices use the reference's FP32 r2 and dp.dv (bit-identical
//      decisions).
//   3. each pair's correction is evaluated in FP32, rounded to an integer
//      of the fixed point (unit = (2 Gmax + Kmax) 2^-40 per pair table) and
//      summed in 64 bits: integer adds are exact, so the sum does not depend
//      on the order in which bodies landed in buckets or lanes found them,
//      and the result is bit-reproducible.
// The all-pairs epilogue adds the correction before its single rounding.
//
// Two passes share the bodies.  contact_kernel gives one warp to each body
// of an ordinary cell.  Crowded buckets (gi_options.dense_min bodies, 256 by
// default, or a quarter of that next to such a cell; e.g. an
// interpenetrating collision remnant with thousands of contacts per body)
// whose bodies all share one cell are sorted by sub-cell and go through
// contact_tile_kernel: a work item is (bucket,
// neighbour bucket, chunk of 128 of its bodies); its CTA stages the
// neighbour bucket in shared memory 128 bodies at a time, each thread
// filters the tile into a hit list and evaluates the law on the hits only,
// and a pair of two dense cells is evaluated once for both bodies.  The
// candidate sets, the pair law and the fixed-point terms are the same on
// both paths and integer addition is exact, so the corrections are
// bit-identical whichever path a body takes.
#include <algorithm>

#include "gi_force_impl.cuh"

namespace gi {

__device__ __forceinline__ int cell_of(float x)
{
    float f = floorf(x);
    f = fminf(fmaxf(f, -1.0e9f), 1.0e9f);  // far debris shares edge cells; NaN -> -1e9
    return (int)f;
}

__device__ __forceinline__ unsigned int bucket_of(int run, int cx, int cy, int cz,
                                                  unsigned int mask)
{
    unsigned int h = (unsigned int)cx * 73856093u;
    h ^= (unsigned int)cy * 19349663u;
    h ^= (unsigned int)cz * 83492791u;
    h ^= (unsigned int)run * 2654435761u;
    h ^= h >> 15;
    return h & mask;
}

// Bucket of every body of every run; histogram of buckets.
__global__ void __launch_bounds__(256)
grid_keys(const float4 *__restrict__ pos, const __grid_constant__ LaunchTable tab,
          unsigned int mask, unsigned int *__restrict__ keys, unsigned int *__restrict__ hist)
{
    const RunDev &R = tab.runs[blockIdx.y];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < R.n; k += gridDim.x * blockDim.x) {
        const int i = R.offset + k;
        const float4 p = pos[i];
        const unsigned int b = bucket_of(blockIdx.y, cell_of(p.x), cell_of(p.y), cell_of(p.z), mask);
        keys[i] = b;
        atomicAdd(&hist[b], 1u);
    }
}

// Exclusive scan of a[0..m), m <= 1024 * 8192, in place.
__global__ void __launch_bounds__(1024) scan_blocks(unsigned int *__restrict__ a, int m,
                                                    unsigned int *__restrict__ sums)
{
    __shared__ unsigned int sh[1024];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const unsigned int v = i < m ? a[i] : 0u;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0u;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < m) a[i] = sh[threadIdx.x] - v;
    if (threadIdx.x == 1023) sums[blockIdx.x] = sh[1023];
}

// Exclusive scan of nb <= 8192 block totals: 8 per thread, then across threads.
__global__ void __launch_bounds__(1024) scan_sums(unsigned int *__restrict__ sums, int nb)
{
    __shared__ unsigned int sh[1024];
    unsigned int loc[8];
    unsigned int tot = 0u;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int i = threadIdx.x * 8 + q;
        loc[q] = i < nb ? sums[i] : 0u;
        tot += loc[q];
    }
    sh[threadIdx.x] = tot;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0u;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    unsigned int run = sh[threadIdx.x] - tot;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int i = threadIdx.x * 8 + q;
        if (i < nb) sums[i] = run;
        run += loc[q];
    }
}

__global__ void __launch_bounds__(1024) scan_add(unsigned int *__restrict__ a, int m,
                                                 const unsigned int *__restrict__ sums)
{
    const int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < m) a[i] += sums[blockIdx.x];
}

// After this, bucket b holds sorted[(b ? cursor[b-1] : 0) .. cursor[b]),
// and spos / svel hold each slot's body state: the contact passes read
// candidates slot by slot, coalesced and without the index hop.
__global__ void __launch_bounds__(256)
grid_scatter(const float4 *__restrict__ pos, const float4 *__restrict__ vel,
             const __grid_constant__ LaunchTable tab, const unsigned int *__restrict__ keys,
             unsigned int *__restrict__ cursor, int *__restrict__ sorted, float4 *__restrict__ spos,
             float4 *__restrict__ svel)
{
    const RunDev &R = tab.runs[blockIdx.y];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < R.n; k += gridDim.x * blockDim.x) {
        const int i = R.offset + k;
        const unsigned int slot = atomicAdd(&cursor[keys[i]], 1u);
        sorted[slot] = i;
        spos[slot] = pos[i];
        svel[slot] = vel[i];
    }
}

// Pair constants of body i against a j of one material: the class row of
// the table and the far-field term of a contact pair.
struct PairRow {
    float G, K, Tband, Tmid, KRmid, KRin;
    float far;  // -(gm_i gm_j) s_far, the clamped far-field coefficient at r2 < 1
};

__device__ __forceinline__ PairRow pair_row(const PairDev &P, bool ife, bool jfe)
{
    const int test = (int)ife + (int)jfe;
    PairRow w;
    w.G = P.G[test];
    w.K = P.K[test];
    w.Tband = P.Tband[test];
    w.Tmid = P.Tmid[test];
    w.KRmid = P.KRmid[test];
    w.KRin = P.KRin[test];
    // every contact pair has r2 < 1, where the all-pairs pass clamps r2 to 1
    const float ri = rsqrt_mufu(1.0f);
    const float s_far = (ri * ri) * ri;
    const float gmi = ife ? P.gm_fe : P.gm_si;
    const float gmj = jfe ? P.gm_fe : P.gm_si;
    w.far = -(gmi * gmj) * s_far;
    return w;
}

__device__ __forceinline__ PairRow select_row(bool jfe, const PairRow &fe, const PairRow &si)
{
    PairRow w;
    w.G = jfe ? fe.G : si.G;
    w.K = jfe ? fe.K : si.K;
    w.Tband = jfe ? fe.Tband : si.Tband;
    w.Tmid = jfe ? fe.Tmid : si.Tmid;
    w.KRmid = jfe ? fe.KRmid : si.KRmid;
    w.KRin = jfe ? fe.KRin : si.KRin;
    w.far = jfe ? fe.far : si.far;
    return w;
}

// Contact correction of one pair with r2 < 1, as a coefficient of dp in
// force units: the reference law's contact force on i, mag dp / r, minus
// the clamped far-field term gm_i gm_j dp the all-pairs pass added.
__device__ __forceinline__ float contact_coef(const PairRow &w, int sep_test, float dx, float dy,
                                              float dz, float r2, float4 vi, float4 vj)
{
    float K = w.K;
    if (!(r2 >= w.Tband)) {
        const float dvx = __fsub_rn(vj.x, vi.x), dvy = __fsub_rn(vj.y, vi.y),
                    dvz = __fsub_rn(vj.z, vi.z);
        const float dpdv = __fmaf_rn(dz, dvz, __fmaf_rn(dx, dvx, __fmul_rn(dy, dvy)));
        // Reference: int inout = dp.dv; KR when inout > 0, i.e. dp.dv >= 1.
        const bool sep = (sep_test == GI_SEP_SIGN) ? (dpdv > 0.0f) : (dpdv >= 1.0f);
        if (sep) K = (r2 >= w.Tmid) ? w.KRmid : w.KRin;
    }
    const float mag = contact_mag(w.G, K, r2);
    // 1 / r: MUFU rsqrt and one Newton-Raphson step (about 1 ulp)
    float invr = rsqrt_mufu(r2);
    invr = invr * __fmaf_rn(-0.5f * r2 * invr, invr, 1.5f);
    return __fmaf_rn(mag, invr, w.far);
}

// contact_coef with j's velocity read (from shared memory) only for pairs
// inside the shell band, where the separation test needs it.  Same
// arithmetic, same result.
__device__ __forceinline__ float contact_coef_at(const PairRow &w, int sep_test, float dx,
                                                 float dy, float dz, float r2, float4 vi,
                                                 const float4 *vj)
{
    float K = w.K;
    if (!(r2 >= w.Tband)) {
        const float4 v = *vj;
        const float dvx = __fsub_rn(v.x, vi.x), dvy = __fsub_rn(v.y, vi.y),
                    dvz = __fsub_rn(v.z, vi.z);
        const float dpdv = __fmaf_rn(dz, dvz, __fmaf_rn(dx, dvx, __fmul_rn(dy, dvy)));
        const bool sep = (sep_test == GI_SEP_SIGN) ? (dpdv > 0.0f) : (dpdv >= 1.0f);
        if (sep) K = (r2 >= w.Tmid) ? w.KRmid : w.KRin;
    }
    const float mag = contact_mag(w.G, K, r2);
    float invr = rsqrt_mufu(r2);
    invr = invr * __fmaf_rn(-0.5f * r2 * invr, invr, 1.5f);
    return __fmaf_rn(mag, invr, w.far);
}

// Fixed-point sums without the FP64 unit.  Each pair term x (FP32, in
// units of the fixed point) is rounded to the nearest integer, ties to
// even, exactly as cvt.rni.s64.f32 would; that instruction issues on the
// FP64 unit, the slowest unit of this GPU, so the terms are split on the
// FP32 pipe instead.  For |x| < 2^45:
//   s = fl(x + 1.5 2^46) is x rounded to a multiple of 2^23 (ulp 2^23) plus
//       1.5 2^46, and stays in [2^46, 2^47], so its bit pattern minus that
//       of 1.5 2^46 is hi = (s - 1.5 2^46) / 2^23;
//   lo = x - hi 2^23 is exact (|lo| <= 2^22), and fl(lo + 1.5 2^23) rounds
//       it to an integer (ulp 1, ties to even), read back the same way.
// round(x) = hi 2^23 + round(lo) because 2^23 is even.  Bit patterns are
// summed mod 2^32 and folded into 64 bits at most every kFixFold terms,
// before the 32-bit sums of hi and lo (each |.| <= 2^22 a term) can wrap.
constexpr float kFixM = 0x1.8p46f;  // 1.5 * 2^46
constexpr float kFixC = 0x1.8p23f;  // 1.5 * 2^23
constexpr float kFixMax = 0x1p45f;  // largest |term| the split takes
constexpr unsigned int kFixFold = 256;
// A pair term is at most 2^40 (1 + 2^-16) units (see fix_in_range).
static_assert(0x1p40f * (1.0f + 0x1p-16f) < kFixMax, "the split must take every pair term");
// kFixFold terms of at most 2^22 each fit the 32-bit pending sums.
static_assert((double)kFixFold * 0x1p22 < 0x1p31, "pending sums must not wrap");

struct FixSum3 {
    long long x, y, z;           // folded sums
    unsigned int hx, hy, hz;     // pending bit-pattern sums of s
    unsigned int lx, ly, lz;     // pending bit-pattern sums of fl(lo + 1.5 2^23)
    unsigned int n;              // pending terms
};

__device__ __forceinline__ void fix_zero(FixSum3 &a)
{
    a.x = a.y = a.z = 0;
    a.hx = a.hy = a.hz = a.lx = a.ly = a.lz = a.n = 0u;
}

__device__ __forceinline__ void fix_split(float x, unsigned int &h, unsigned int &l)
{
    const float s = __fadd_rn(x, kFixM);
    const float lo = __fsub_rn(x, __fsub_rn(s, kFixM));
    h += __float_as_uint(s);
    l += __float_as_uint(__fadd_rn(lo, kFixC));
}

__device__ __forceinline__ long long fix_value(unsigned int h, unsigned int l, unsigned int n)
{
    const int hi = (int)(h - n * __float_as_uint(kFixM));
    const int lo = (int)(l - n * __float_as_uint(kFixC));
    return (long long)hi * (1ll << 23) + lo;
}

__device__ __forceinline__ void fix_fold(FixSum3 &a)
{
    a.x += fix_value(a.hx, a.lx, a.n);
    a.y += fix_value(a.hy, a.ly, a.n);
    a.z += fix_value(a.hz, a.lz, a.n);
    a.hx = a.hy = a.hz = a.lx = a.ly = a.lz = a.n = 0u;
}

// The split is exact for every term of a pair with a normal r2: there
// 1 / r is finite, |d| <= r (up to rounding), so |c d| <= (|mag| + G m m) /
// unit <= 2^40 (1 + 2^-16) < kFixMax, the fixed-point unit being
// (2 Gmax + Kmax) 2^-40.  Coincident bodies (r2 = 0), a denormal r2 (the
// MUFU rsqrt flushes it to zero) or NaN take the hardware conversion,
// which rounds the same way; so the choice never changes a result.
__device__ __forceinline__ bool fix_in_range(float r2) { return r2 >= 0x1p-126f; }

// Adds round(c dx), round(c dy), round(c dz) for a pair of squared
// distance r2 (see fix_in_range); x and y in packed FP32x2 instructions,
// with the roundings of fix_split (s = fl(t + M); lo = fl(t - fl(s - M)),
// here as fma(fl(s - M), -1, t); fl(lo + C)).  FOLD: fold when kFixFold
// terms are pending (a caller that adds fewer terms between its own folds
// passes false).
template <bool FOLD = true>
__device__ __forceinline__ void fix_add3(FixSum3 &a, float c, float dx, float dy, float dz,
                                         float r2)
{
    const float2 txy = __fmul2_rn(make_float2(c, c), make_float2(dx, dy));
    const float tz = __fmul_rn(c, dz);
    if (fix_in_range(r2)) {
        const float2 s = __fadd2_rn(txy, make_float2(kFixM, kFixM));
        const float2 lo = __ffma2_rn(__fadd2_rn(s, make_float2(-kFixM, -kFixM)),
                                     make_float2(-1.0f, -1.0f), txy);
        const float2 l = __fadd2_rn(lo, make_float2(kFixC, kFixC));
        a.hx += __float_as_uint(s.x);
        a.hy += __float_as_uint(s.y);
        a.lx += __float_as_uint(l.x);
        a.ly += __float_as_uint(l.y);
        fix_split(tz, a.hz, a.lz);
        ++a.n;
        if (FOLD && a.n == kFixFold) fix_fold(a);
    } else {
        a.x += __float2ll_rn(txy.x);
        a.y += __float2ll_rn(txy.y);
        a.z += __float2ll_rn(tz);
    }
}

// Pair form of fix_add3 for an unordered pair evaluated once: adds
// round(c d) to body i's sums and -round(c d), exactly the term body j's own
// evaluation would give (dp and dv change sign exactly, c is symmetric, and
// rounding to nearest even is odd-symmetric), to the shared sums js[.][k]
// of j's staged slot: true values mod 2^32, hi in js[0..2], lo in js[3..5].
// A term out of the split's range goes to j's global sums directly.  The
// caller folds (at most kFixFold terms between its folds).
__device__ __forceinline__ void fix_add3_pair(FixSum3 &a, unsigned int (*js)[128], int k,
                                              long long *dj, float c, float dx, float dy, float dz,
                                              float r2)
{
    const float2 txy = __fmul2_rn(make_float2(c, c), make_float2(dx, dy));
    const float tz = __fmul_rn(c, dz);
    if (fix_in_range(r2)) {
        const float2 s = __fadd2_rn(txy, make_float2(kFixM, kFixM));
        const float2 lo = __ffma2_rn(__fadd2_rn(s, make_float2(-kFixM, -kFixM)),
                                     make_float2(-1.0f, -1.0f), txy);
        const float2 l = __fadd2_rn(lo, make_float2(kFixC, kFixC));
        const float sz = __fadd_rn(tz, kFixM);
        const float lz = __fadd_rn(__fsub_rn(tz, __fsub_rn(sz, kFixM)), kFixC);
        const unsigned int sb[3] = {__float_as_uint(s.x), __float_as_uint(s.y), __float_as_uint(sz)};
        const unsigned int lb[3] = {__float_as_uint(l.x), __float_as_uint(l.y), __float_as_uint(lz)};
        a.hx += sb[0]; a.hy += sb[1]; a.hz += sb[2];
        a.lx += lb[0]; a.ly += lb[1]; a.lz += lb[2];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            atomicAdd(&js[d][k], __float_as_uint(kFixM) - sb[d]);
            atomicAdd(&js[3 + d][k], __float_as_uint(kFixC) - lb[d]);
        }
        ++a.n;
    } else {
        const long long vx = __float2ll_rn(txy.x), vy = __float2ll_rn(txy.y),
                        vz = __float2ll_rn(tz);
        a.x += vx;
        a.y += vy;
        a.z += vz;
        unsigned long long *d = reinterpret_cast<unsigned long long *>(dj);
        atomicAdd(d + 0, 0ull - (unsigned long long)vx);
        atomicAdd(d + 1, 0ull - (unsigned long long)vy);
        atomicAdd(d + 2, 0ull - (unsigned long long)vz);
    }
}

// Adds the shared j-side sums of slot t to body j's correction and clears them.
__device__ __forceinline__ void flush_slot(unsigned int (*js)[128], int t, int j, long long *delta)
{
    long long v[3];
    bool any = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        v[d] = (long long)(int)js[d][t] * (1ll << 23) + (int)js[3 + d][t];
        any |= v[d] != 0;
        js[d][t] = 0u;
        js[3 + d][t] = 0u;
    }
    if (any) {
        unsigned long long *p = reinterpret_cast<unsigned long long *>(delta + 3 * (size_t)j);
        atomicAdd(p + 0, (unsigned long long)v[0]);
        atomicAdd(p + 1, (unsigned long long)v[1]);
        atomicAdd(p + 2, (unsigned long long)v[2]);
    }
}

// A bucket whose bodies share one cell takes the tiled path when it holds
// at least tab.dense_min bodies (256 unless set), or at least a quarter of
// that next to a cell that does: near a crowded remnant its bodies have
// enough contacts to pay the tiled path's fixed costs per item, while the
// cores of settled bodies (cells of tens to a few hundred bodies, ~20
// contacts a body) stay on the warp path.  Either bound is at least
// kDenseFloor, which bounds the item count.  Bucket state bits: 1 = mixed
// cells (stays on the warp path), 2 = tiled.
// (kDenseFloor itself lives in gi_internal.h: it sizes the scratch.)
constexpr unsigned int kMixed = 1u, kTiled = 2u;

__host__ __device__ __forceinline__ unsigned int dense_hi(unsigned int dmin)
{
    return dmin > kDenseFloor ? dmin : kDenseFloor;
}

__host__ __device__ __forceinline__ unsigned int dense_lo(unsigned int dmin)
{
    return dmin / 4u > kDenseFloor ? dmin / 4u : kDenseFloor;
}

// Contact correction of body i (run r) by one warp.  Lanes 0..26 look up
// the 27 neighbour buckets at once (one memory round trip; a bucket that
// two neighbour cells share is kept once), a warp scan lays their bodies
// end to end, and the warp then filters that list 64 candidates at a time
// into the shared hit list q (96 slots), which it evaluates 32 at a time.
__device__ __forceinline__ void contact_body_warp(const float4 *__restrict__ pos,
                                                  const float4 *__restrict__ vel,
                                                  const float4 *__restrict__ spos,
                                                  const float4 *__restrict__ svel,
                                                  const unsigned int *__restrict__ cursor,
                                                  const int *__restrict__ sorted, unsigned int mask,
                                                  long long *__restrict__ delta, const RunDev &R,
                                                  const PairDev &P, int sep_test, int r, int i,
                                                  int lane, unsigned int *q)
{
    const int rbeg = R.offset, rend = R.offset + R.n, sw = R.offset + R.nfe;
    const float4 pi = __ldg(&pos[i]);
    const int cx = cell_of(pi.x), cy = cell_of(pi.y), cz = cell_of(pi.z);

    unsigned int b = 0xffffffffu, beg = 0u, cnt = 0u;
    if (lane < 27) {
        const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
        b = bucket_of(r, cx + ox, cy + oy, cz + oz, mask);
    }
    const unsigned int same = __match_any_sync(0xffffffffu, b);
    const bool first = (same & ((1u << lane) - 1u)) == 0u;
    if (lane < 27 && first) {
        beg = b ? __ldg(&cursor[b - 1]) : 0u;
        cnt = __ldg(&cursor[b]) - beg;
    }
    // inclusive scan of cnt over the warp
    unsigned int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const unsigned int total = __shfl_sync(0xffffffffu, incl, 31);
    const unsigned int excl = incl - cnt;

    const float inv_unit = P.inv_unit;
    const PairRow row_fe = pair_row(P, i < sw, true), row_si = pair_row(P, i < sw, false);
    const float4 vi = __ldg(&vel[i]);
    const float nan = __int_as_float(0x7fffffff);
    const unsigned int below = (1u << lane) - 1u;
    FixSum3 acc;
    fix_zero(acc);
    // Contact law on queued hits, one per lane (lanes >= n idle): slots
    // q[base .. base + n).
    const auto drain = [&](unsigned int base, unsigned int n) {
        if ((unsigned int)lane >= n) return;
        const unsigned int slot = q[base + lane];
        const int j = __ldg(&sorted[slot]);
        if (j == i || j < rbeg || j >= rend) return;  // the body itself, or another run's body
        const float4 pj = __ldg(&spos[slot]), vj = __ldg(&svel[slot]);
        const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
        const float c =
            contact_coef(select_row(j < sw, row_fe, row_si), sep_test, dx, dy, dz, r2, vi, vj) *
            inv_unit;
        fix_add3(acc, c, dx, dy, dz, r2);
    };
    // 64 candidates a pass, two per lane, so that each lane has two
    // independent loads in flight.  Slots within r2 < 1 are queued in the
    // warp's shared list q and evaluated 32 at a time, so the contact law
    // runs on full warps however sparse the hits.
    unsigned int nq = 0;  // queued hits, the same in every lane
    for (unsigned int base = 0; base < total; base += 64) {
        unsigned int t[2] = {base + lane, base + 32 + lane};
        // the lane whose range [excl, incl) holds t: last lane with excl <= t
        int src[2] = {0, 0};
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const unsigned int e = __shfl_sync(0xffffffffu, excl, src[u] + step);
                if (src[u] + step < 32 && e <= t[u]) src[u] += step;
            }
        }
        unsigned int slot[2];
        float4 pj[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const unsigned int sb = __shfl_sync(0xffffffffu, beg, src[u]);
            const unsigned int se = __shfl_sync(0xffffffffu, excl, src[u]);
            slot[u] = sb + (t[u] - se);
            pj[u] = t[u] < total ? __ldg(&spos[slot[u]]) : make_float4(nan, nan, nan, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const float dx = pj[u].x - pi.x, dy = pj[u].y - pi.y, dz = pj[u].z - pi.z;
            const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
            const bool hit = r2 < 1.0f;
            const unsigned int m = __ballot_sync(0xffffffffu, hit);
            if (hit) q[nq + __popc(m & below)] = slot[u];
            nq += __popc(m);
        }
        __syncwarp();
        while (nq >= 32u) {
            nq -= 32u;
            drain(nq, 32u);
            __syncwarp();  // the slots are read before the queue refills
        }
    }
    drain(0u, nq);
    fix_fold(acc);
    long long ax = acc.x, ay = acc.y, az = acc.z;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ax += __shfl_down_sync(0xffffffffu, ax, off);
        ay += __shfl_down_sync(0xffffffffu, ay, off);
        az += __shfl_down_sync(0xffffffffu, az, off);
    }
    if (lane == 0) {
        delta[3 * (size_t)i + 0] = ax;
        delta[3 * (size_t)i + 1] = ay;
        delta[3 * (size_t)i + 2] = az;
    }
}

__device__ __forceinline__ unsigned int bucket_size(const unsigned int *__restrict__ cursor,
                                                    unsigned int b)
{
    return __ldg(&cursor[b]) - (b ? __ldg(&cursor[b - 1]) : 0u);
}

// One warp per body of the run blockIdx.y; bodies of tiled buckets are left
// to contact_tile_kernel.
__global__ void __launch_bounds__(256)
contact_kernel(const float4 *__restrict__ pos, const float4 *__restrict__ vel,
               const float4 *__restrict__ spos, const float4 *__restrict__ svel,
               const unsigned int *__restrict__ cursor, const int *__restrict__ sorted,
               const unsigned int *__restrict__ keys, const unsigned int *__restrict__ state,
               unsigned int mask, long long *__restrict__ delta,
               const __grid_constant__ LaunchTable tab)
{
    __shared__ unsigned int hitq[8][96];  // per warp (up to 8): queued hit slots (up to 31 + 64)
    const RunDev &R = tab.runs[blockIdx.y];
    const int lane = threadIdx.x & 31;
    const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k >= R.n) return;  // whole warp leaves together
    const int i = R.offset + k;
    if (state[__ldg(&keys[i])] & kTiled) return;
    contact_body_warp(pos, vel, spos, svel, cursor, sorted, mask, delta, R, tab.params[R.param],
                      tab.sep_test, blockIdx.y, i, lane, hitq[threadIdx.x >> 5]);
}

// Pass 1, one thread per body of the run blockIdx.y: for bodies of buckets
// that may be tiled (at least dense_lo bodies), clear the correction (the
// tiled path adds into it; the warp path overwrites it) and mark the bucket
// mixed when the body's cell or run differs from the bucket's first body.
__global__ void __launch_bounds__(256)
dense_check_kernel(const float4 *__restrict__ pos, const __grid_constant__ LaunchTable tab,
                   const unsigned int *__restrict__ keys, const unsigned int *__restrict__ cursor,
                   const int *__restrict__ sorted, unsigned int dmin, unsigned int *state,
                   long long *__restrict__ delta)
{
    const RunDev &R = tab.runs[blockIdx.y];
    const unsigned int lo = dense_lo(dmin);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < R.n; k += gridDim.x * blockDim.x) {
        const int i = R.offset + k;
        const unsigned int b = keys[i];
        if (bucket_size(cursor, b) < lo) continue;
        delta[3 * (size_t)i + 0] = 0;
        delta[3 * (size_t)i + 1] = 0;
        delta[3 * (size_t)i + 2] = 0;
        const int j0 = sorted[b ? cursor[b - 1] : 0u];
        if (j0 == i) continue;
        bool mixed = j0 < R.offset || j0 >= R.offset + R.n;
        if (!mixed) {
            const float4 p = pos[i], q = pos[j0];
            mixed = cell_of(p.x) != cell_of(q.x) || cell_of(p.y) != cell_of(q.y) ||
                    cell_of(p.z) != cell_of(q.z);
        }
        if (mixed) atomicOr(&state[b], kMixed);
    }
}

__device__ __forceinline__ int run_of_body(const LaunchTable &tab, int i)
{
    for (int q = 0; q < tab.nruns; ++q)
        if (i >= tab.runs[q].offset && i < tab.runs[q].offset + tab.runs[q].n) return q;
    return 0;
}

// Work item of the tiled path, self-contained so that the tile kernel reads
// it in one load, with no hop through the bucket bounds:
//   x = first slot of the chunk of (up to) 128 bodies of bucket b,
//   y = first slot of the neighbour bucket nb to stage (the chunk's own
//       first slot when nb == b, else the start of nb),
//   z = end of nb,
//   w = run | cost class << 8 | pair << 12 | self << 13 | bodies of the
//       chunk << 16.
// The cost class is the number of 128-body tiles the item stages, minus
// one, capped at kItemClasses - 1; pair: nb is tiled too (each pair is
// evaluated once for both bodies); self: nb == b.
// (kItemClasses lives in gi_internal.h.)

// Counters of the tiled path, in one block of kCtrWords words cleared per
// pass: item count, tiled-bucket count, queue head, then the items per cost
// class and the fill of each class while ordering.
constexpr int kCtrItems = 0, kCtrTiled = 1, kCtrHead = 2, kCtrClass = 4,
              kCtrFill = 4 + (int)kItemClasses;
static_assert(kCtrFill + (int)kItemClasses == kCtrWords, "tiled-path counter block");

// Pass 2, one thread per bucket: a crowded bucket of one cell (see
// dense_hi, dense_lo) becomes tiled and is listed in tiled[0 .. *ntiled).
__global__ void __launch_bounds__(256)
dense_mark_kernel(const float4 *__restrict__ pos, const __grid_constant__ LaunchTable tab,
                  const unsigned int *__restrict__ cursor, const int *__restrict__ sorted,
                  unsigned int m, unsigned int mask, unsigned int dmin, unsigned int *state,
                  unsigned int *__restrict__ tiled, unsigned int *__restrict__ ntiled)
{
    const unsigned int hi = dense_hi(dmin), lo = dense_lo(dmin);
    for (unsigned int b = blockIdx.x * blockDim.x + threadIdx.x; b < m; b += gridDim.x * blockDim.x) {
        const unsigned int n = bucket_size(cursor, b);
        if (n < lo || (state[b] & kMixed)) continue;
        bool crowded = n >= hi;
        if (!crowded) {  // a neighbour cell of at least hi bodies?
            const int j0 = sorted[b ? cursor[b - 1] : 0u];
            const int r = run_of_body(tab, j0);
            const float4 p = pos[j0];
            const int cx = cell_of(p.x), cy = cell_of(p.y), cz = cell_of(p.z);
            for (int q = 0; q < 27 && !crowded; ++q)
                crowded = bucket_size(cursor, bucket_of(r, cx + q % 3 - 1, cy + (q / 3) % 3 - 1,
                                                        cz + q / 9 - 1, mask)) >= hi;
        }
        if (!crowded) continue;
        state[b] = kTiled;
        tiled[atomicAdd(ntiled, 1u)] = b;
    }
}

// Pass 4, one warp per tiled bucket b: an item per (chunk of 128 of its
// bodies, distinct non-empty neighbour bucket nb).  Lanes 0..26 look up
// the 27 neighbour buckets at once; a bucket that two neighbour cells
// share is kept once.  A pair of tiled buckets is listed once, from the
// lower bucket number (nb >= b): its item evaluates each contact pair once
// for both bodies.  A bucket that is not tiled gets its own sums from
// contact_kernel, so its item adds to b's bodies only.  Items are written
// chunk by chunk, neighbours in offset order within a chunk.
__global__ void __launch_bounds__(256)
dense_items_kernel(const float4 *__restrict__ pos, const __grid_constant__ LaunchTable tab,
                   const unsigned int *__restrict__ cursor, const int *__restrict__ sorted,
                   unsigned int mask, const unsigned int *__restrict__ state,
                   const unsigned int *__restrict__ tiled, unsigned int *__restrict__ ctr,
                   uint4 *__restrict__ items)
{
    const unsigned int *ntiled = ctr + kCtrTiled;
    unsigned int *nitems = ctr + kCtrItems;
    const unsigned int lane = threadIdx.x & 31u;
    const unsigned int total = *ntiled;
    const unsigned int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (unsigned int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < total; w += nwarps) {
        const unsigned int b = tiled[w];
        const unsigned int cnt = bucket_size(cursor, b);
        const int j0 = sorted[b ? cursor[b - 1] : 0u];
        const int r = run_of_body(tab, j0);
        const float4 p = pos[j0];
        unsigned int nbq = 0xffffffffu;  // no bucket: lanes 27..31
        if (lane < 27u)
            nbq = bucket_of(r, cell_of(p.x) + (int)(lane % 3u) - 1, cell_of(p.y) + (int)(lane / 3u % 3u) - 1,
                            cell_of(p.z) + (int)(lane / 9u) - 1, mask);
        const unsigned int same = __match_any_sync(0xffffffffu, nbq);
        bool keep = false;
        if (lane < 27u && (same & ((1u << lane) - 1u)) == 0u) {
            const bool other_side = (state[nbq] & kTiled) && nbq < b;
            keep = !other_side && bucket_size(cursor, nbq) > 0u;
        }
        const unsigned int km = __ballot_sync(0xffffffffu, keep);
        const unsigned int nq = __popc(km), nch = (cnt + 127u) / 128u;
        unsigned int at = 0u;
        if (lane == 0u) at = atomicAdd(nitems, nch * nq);
        at = __shfl_sync(0xffffffffu, at, 0);
        if (keep) {
            const unsigned int rank = __popc(km & ((1u << lane) - 1u));
            const unsigned int bbeg = b ? cursor[b - 1] : 0u;
            const unsigned int nbeg = nbq ? cursor[nbq - 1] : 0u, nend = cursor[nbq];
            const unsigned int flags = (unsigned int)r | ((state[nbq] & kTiled) ? 1u << 12 : 0u) |
                                       (nbq == b ? 1u << 13 : 0u);
            for (unsigned int c = 0; c < nch; ++c) {
                const unsigned int s0 = bbeg + 128u * c;
                const unsigned int first = nbq == b ? s0 : nbeg;
                const unsigned int cls = min((nend - first + 127u) / 128u, kItemClasses) - 1u;
                const unsigned int ni = min(128u, bbeg + cnt - s0);
                items[at + c * nq + rank] = make_uint4(s0, first, nend, flags | cls << 8 | ni << 16);
                atomicAdd(&ctr[kCtrClass + cls], 1u);
            }
        }
    }
}

// Pass 5: the items, ordered by cost class, most tiles first (a counting
// sort over the classes), so that the tile kernel's queue hands out the
// longest items first and its CTAs finish together.  Order within a class
// is arbitrary; the sums do not depend on it.
__global__ void __launch_bounds__(256)
dense_order_kernel(const uint4 *__restrict__ raw, unsigned int *__restrict__ ctr,
                   uint4 *__restrict__ items)
{
    __shared__ unsigned int base[kItemClasses];
    if (threadIdx.x < kItemClasses) {
        unsigned int b = 0;
        for (unsigned int c = kItemClasses - 1; c > threadIdx.x; --c) b += ctr[kCtrClass + c];
        base[threadIdx.x] = b;
    }
    __syncthreads();
    const unsigned int total = ctr[kCtrItems];
    for (unsigned int w = blockIdx.x * blockDim.x + threadIdx.x; w < total;
         w += gridDim.x * blockDim.x) {
        const uint4 it = raw[w];
        const unsigned int cls = (it.w >> 8) & (kItemClasses - 1u);
        items[base[cls] + atomicAdd(&ctr[kCtrFill + cls], 1u)] = it;
    }
}

// Sub-cell of a body inside its unit cell: 4 x 4 x 4 sub-cells of D/4,
// numbered in Morton order.
__device__ __forceinline__ unsigned int subcell_of(float4 p)
{
    const auto q = [](float x) {
        const int s = (int)((x - floorf(x)) * 4.0f);  // NaN -> 0
        return (unsigned int)min(max(s, 0), 3);
    };
    const unsigned int sx = q(p.x), sy = q(p.y), sz = q(p.z);
    return (sx & 1u) | (sy & 1u) << 1 | (sz & 1u) << 2 | (sx >> 1) << 3 | (sy >> 1) << 4 |
           (sz >> 1) << 5;
}

// Buckets of up to kSortCap bodies are sorted in shared memory.
constexpr unsigned int kSortCap = 8192;

// Pass 3, one CTA per tiled bucket: reorder the bucket's slots by sub-cell
// (counting sort), so that the 32 bodies of a warp, and the 32 of a
// staged block, sit close together.  Only the order within the bucket
// changes; the contact sums are exact integer sums, so the forces do not
// depend on it.  A bucket above kSortCap keeps its order.
__global__ void __launch_bounds__(256)
dense_sort_kernel(const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                  const unsigned int *__restrict__ cursor, int *__restrict__ sorted,
                  float4 *__restrict__ spos, float4 *__restrict__ svel,
                  const unsigned int *__restrict__ tiled, const unsigned int *__restrict__ ntiled)
{
    __shared__ int sidx[kSortCap];
    __shared__ unsigned char skey[kSortCap];
    __shared__ unsigned int cnt[64];
    const unsigned int total = *ntiled;
    for (unsigned int w = blockIdx.x; w < total; w += gridDim.x) {
        const unsigned int b = tiled[w];
        const unsigned int beg = b ? cursor[b - 1] : 0u, n = cursor[b] - beg;
        if (n > kSortCap) continue;  // the same for every thread of the CTA
        __syncthreads();  // the previous bucket is written out
        if (threadIdx.x < 64) cnt[threadIdx.x] = 0u;
        __syncthreads();
        for (unsigned int u = threadIdx.x; u < n; u += blockDim.x) {
            const int j = sorted[beg + u];
            const unsigned int k = subcell_of(pos[j]);
            sidx[u] = j;
            skey[u] = (unsigned char)k;
            atomicAdd(&cnt[k], 1u);
        }
        __syncthreads();
        if (threadIdx.x < 32) {  // exclusive scan of the 64 counts, two per lane
            const unsigned int lane = threadIdx.x;
            const unsigned int c0 = cnt[2 * lane], c1 = cnt[2 * lane + 1];
            unsigned int incl = c0 + c1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned int v = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int)lane >= o) incl += v;
            }
            const unsigned int excl = incl - c0 - c1;
            cnt[2 * lane] = excl;
            cnt[2 * lane + 1] = excl + c0;
        }
        __syncthreads();
        for (unsigned int u = threadIdx.x; u < n; u += blockDim.x) {
            const int j = sidx[u];
            const unsigned int slot = beg + atomicAdd(&cnt[skey[u]], 1u);
            sorted[slot] = j;
            spos[slot] = pos[j];
            svel[slot] = vel[j];
        }
    }
}

// Bounding box of the non-empty lanes of a warp (lo = +inf, hi = -inf for
// an empty lane), returned to every lane.  fminf / fmaxf drop NaN.
__device__ __forceinline__ void warp_box(float3 &lo, float3 &hi)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo.x = fminf(lo.x, __shfl_xor_sync(0xffffffffu, lo.x, o));
        lo.y = fminf(lo.y, __shfl_xor_sync(0xffffffffu, lo.y, o));
        lo.z = fminf(lo.z, __shfl_xor_sync(0xffffffffu, lo.z, o));
        hi.x = fmaxf(hi.x, __shfl_xor_sync(0xffffffffu, hi.x, o));
        hi.y = fmaxf(hi.y, __shfl_xor_sync(0xffffffffu, hi.y, o));
        hi.z = fmaxf(hi.z, __shfl_xor_sync(0xffffffffu, hi.z, o));
    }
}

// Lower bound, in the rounding of the pair filter, of the FP32 r2 of every
// pair between two boxes.  Per axis, |fl(pj - pi)| >= fl(gap) because
// rounding is monotone, and the sum of squares below has the form of the
// filter's, so a result >= 1 proves that no pair passes r2 < 1.  A NaN term
// (inf - inf) is dropped by fmaxf; each remaining term bounds the finite
// pairs, and pairs with a non-finite coordinate never pass the filter.
__device__ __forceinline__ float box_gap2(float3 ilo, float3 ihi, float3 jlo, float3 jhi)
{
    const float gx = fmaxf(fmaxf(__fsub_rn(jlo.x, ihi.x), __fsub_rn(ilo.x, jhi.x)), 0.0f);
    const float gy = fmaxf(fmaxf(__fsub_rn(jlo.y, ihi.y), __fsub_rn(ilo.y, jhi.y)), 0.0f);
    const float gz = fmaxf(fmaxf(__fsub_rn(jlo.z, ihi.z), __fsub_rn(ilo.z, jhi.z)), 0.0f);
    return __fmaf_rn(gz, gz, __fmaf_rn(gx, gx, __fmul_rn(gy, gy)));
}

// Shared-memory position of staged slot k (0..127).  Lanes walking their
// hit lists (ascending slots) from staggered starts read slots about 4
// apart; this layout puts such slots in distinct banks, for the 16-byte
// staged bodies and for the 4-byte j-side sums alike.
__device__ __forceinline__ int swz(int k) { return ((k & 3) << 5) | (k >> 2); }

// The contact law on one thread's hits of a staged tile (slots my[0 .. nh)),
// starting at the (lane / 32)-th part of the list so that lanes with alike
// lists (neighbouring bodies) rarely hit one slot's shared sums at once.
// PAIR: the pair's j-side term goes to the slot's shared sums too.  MIXED:
// the tile holds Fe bodies, so the pair-class row is chosen per hit; a tile
// of Si bodies alone (most of them: Fe is the small core) uses row_si.
template <bool PAIR, bool MIXED>
__device__ __forceinline__ void tile_hits(FixSum3 &acc, const unsigned char *my, int nh, int lane,
                                          const float4 *sp, const float4 *sv,
                                          unsigned int (*js)[128], long long *delta, float4 pi,
                                          float4 vi, const PairRow &row_fe, const PairRow &row_si,
                                          int sw, int sep_test, float inv_unit)
{
    const float2 npxy = make_float2(-pi.x, -pi.y);
    int h = (lane * nh) >> 5;
    for (int n = 0; n < nh; ++n) {
        const int k = swz(my[h]);  // shared-memory position of the slot
        h = h + 1 == nh ? 0 : h + 1;
        const float4 pj = sp[k];
        const int j = __float_as_int(pj.w);  // never i: b and nb differ, or k > t
        const float2 dxy = __fadd2_rn(make_float2(pj.x, pj.y), npxy);
        const float dx = dxy.x, dy = dxy.y, dz = pj.z - pi.z;
        const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
        const float c = contact_coef_at(MIXED ? select_row(j < sw, row_fe, row_si) : row_si,
                                        sep_test, dx, dy, dz, r2, vi, &sv[k]) *
                        inv_unit;
        if (PAIR) fix_add3_pair(acc, js, k, delta + 3 * (size_t)j, c, dx, dy, dz, r2);
        else fix_add3<false>(acc, c, dx, dy, dz, r2);
    }
    // at most 128 hits a tile: fold before kFixFold terms can be pending
    if (acc.n >= kFixFold - 128u) fix_fold(acc);
}

// Items come from a queue, longest first.  For an item the CTA holds up to
// 128 bodies of the bucket b (one per thread, all in one cell), stages the
// neighbour bucket nb in shared memory 128 bodies at a time, and each
// thread collects the tile slots within r2 < 1 of its body before
// evaluating the contact law on those alone.  A warp skips each staged
// block of 32 bodies whose bounding box is provably out of reach of its own
// bodies' box.  When nb is tiled too, each pair is evaluated once for both
// bodies: the item covers nb's tiles from the chunk's own slots on (all of
// them when nb != b; within the chunk's own tile only slots above the
// thread's), and the staged bodies' shared sums go into their corrections
// with 64-bit global atomics once per tile.
// 72 registers: 7 CTAs of 128 threads per SM, with no spills.
__global__ void __maxnreg__(72)
contact_tile_kernel(const float4 *__restrict__ spos, const float4 *__restrict__ svel,
                    const unsigned int *__restrict__ cursor, const int *__restrict__ sorted,
                    const unsigned int *__restrict__ state, long long *__restrict__ delta,
                    const __grid_constant__ LaunchTable tab, const uint4 *__restrict__ items,
                    unsigned int *__restrict__ ctr)
{
    constexpr int kStride = 132;  // bytes per hit list row: rows start in distinct banks
    __shared__ float4 sp[128];    // x, y, z, body index (bits); NaN xyz outside the run
    __shared__ float4 sv[128];
    __shared__ float3 blo[4], bhi[4];  // box of each staged block of 32
    __shared__ unsigned int js[6][128];  // j-side sums of the staged slots (pair items)
    __shared__ unsigned char hits[128 * kStride];
    __shared__ unsigned int s_w;  // the item to take next
    const unsigned int total = ctr[kCtrItems];
    const int t = threadIdx.x;
    const int tz = swz(t);  // where this thread stages its slot
    const int lane = t & 31, warp = t >> 5;
    const float kInf = __int_as_float(0x7f800000);
    unsigned char *my = hits + t * kStride;
#pragma unroll
    for (int d = 0; d < 6; ++d) js[d][t] = 0u;
    // Thread 0 takes the next item from the queue when the current one
    // reaches its last tile: the atomic's latency hides behind that tile,
    // and the CTA still takes items close to the queue's longest-first order.
    if (t == 0) s_w = atomicAdd(&ctr[kCtrHead], 1u);
    __syncthreads();
    for (;;) {
        const unsigned int w = s_w;
        if (w >= total) break;
        const uint4 rec = items[w];
        unsigned int nw = 0u;  // thread 0: the next item
        const unsigned int s0 = rec.x, first = rec.y, nend = rec.z;
        const unsigned int ni = rec.w >> 16;
        const bool pair = (rec.w >> 12) & 1u, self = (rec.w >> 13) & 1u;
        const bool valid = (unsigned int)t < ni;
        const RunDev &R = tab.runs[rec.w & 0xffu];
        const int rbeg = R.offset, rend = R.offset + R.n, sw = R.offset + R.nfe;
        const float inv_unit = tab.params[R.param].inv_unit;
        const int i = valid ? sorted[s0 + t] : -1;
        const float4 pi = valid ? spos[s0 + t] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 vi = valid ? svel[s0 + t] : make_float4(0.f, 0.f, 0.f, 0.f);
        const PairRow row_fe = pair_row(tab.params[R.param], i < sw, true);
        const PairRow row_si = pair_row(tab.params[R.param], i < sw, false);
        float3 ilo = valid ? make_float3(pi.x, pi.y, pi.z) : make_float3(kInf, kInf, kInf);
        float3 ihi = valid ? make_float3(pi.x, pi.y, pi.z) : make_float3(-kInf, -kInf, -kInf);
        warp_box(ilo, ihi);
        FixSum3 acc;
        fix_zero(acc);
        for (unsigned int base = first; base < nend; base += 128u) {
            __syncthreads();  // the previous tile is consumed
            if (pair && base != first) flush_slot(js, tz, __float_as_int(sp[tz].w), delta);
            if (t == 0 && base + 128u >= nend) nw = atomicAdd(&ctr[kCtrHead], 1u);
            const unsigned int u = base + (unsigned int)t;
            float3 lo = make_float3(kInf, kInf, kInf), hi = make_float3(-kInf, -kInf, -kInf);
            bool fe_slot = false;  // the staged body is of the run's Fe core
            if (u < nend) {
                const int j = sorted[u];
                if (j >= rbeg && j < rend) {
                    fe_slot = j < sw;
                    const float4 q = spos[u];
                    sp[tz] = make_float4(q.x, q.y, q.z, __int_as_float(j));
                    sv[tz] = svel[u];
                    lo = hi = make_float3(q.x, q.y, q.z);
                } else {  // another run's body, in a bucket shared by hashing: never a hit
                    const float nan = __int_as_float(0x7fffffff);
                    sp[tz] = make_float4(nan, nan, nan, __int_as_float(j));
                }
            }
            warp_box(lo, hi);
            if (lane == 0) {
                blo[warp] = lo;
                bhi[warp] = hi;
            }
            // does any staged body of the run belong to the Fe core?
            const int mixed = __syncthreads_or(fe_slot);
            if (!valid) continue;
            const int cnt = (int)min(128u, nend - base);
            const int kmin = (self && base == first) ? t + 1 : 0;  // own tile: each pair once
            int nh = 0;
            for (int s = 0; s < 4 && 32 * s < cnt; ++s) {
                if (box_gap2(ilo, ihi, blo[s], bhi[s]) >= 1.0f) continue;  // the same for the warp
                const int k1 = min(cnt, 32 * s + 32);
                for (int k = 32 * s; k < k1; k += 4) {  // swz(k + c) = 32 c + k / 4
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        if (k + c >= k1) break;
                        const float4 pj = sp[32 * c + (k >> 2)];
                        const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
                        const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
                        if (r2 < 1.0f && k + c >= kmin) my[nh++] = (unsigned char)(k + c);
                    }
                }
            }
            if (pair) {
                if (mixed)
                    tile_hits<true, true>(acc, my, nh, lane, sp, sv, js, delta, pi, vi, row_fe,
                                          row_si, sw, tab.sep_test, inv_unit);
                else
                    tile_hits<true, false>(acc, my, nh, lane, sp, sv, js, delta, pi, vi, row_fe,
                                           row_si, sw, tab.sep_test, inv_unit);
            } else {
                if (mixed)
                    tile_hits<false, true>(acc, my, nh, lane, sp, sv, js, delta, pi, vi, row_fe,
                                           row_si, sw, tab.sep_test, inv_unit);
                else
                    tile_hits<false, false>(acc, my, nh, lane, sp, sv, js, delta, pi, vi, row_fe,
                                            row_si, sw, tab.sep_test, inv_unit);
            }
        }
        __syncthreads();  // the last tile's j-side sums are complete; s_w is read
        if (pair) flush_slot(js, tz, __float_as_int(sp[tz].w), delta);
        if (t == 0) s_w = nw;
        __syncthreads();  // the next item's index is visible
        fix_fold(acc);
        const long long ax = acc.x, ay = acc.y, az = acc.z;
        if (valid && (ax | ay | az)) {
            unsigned long long *d = reinterpret_cast<unsigned long long *>(delta + 3 * (size_t)i);
            atomicAdd(d + 0, (unsigned long long)ax);
            atomicAdd(d + 1, (unsigned long long)ay);
            atomicAdd(d + 2, (unsigned long long)az);
        }
    }
}

}  // namespace gi

// gi_grid_buckets and gi_grid_words (the scratch layout) are in gi_internal.h.

cudaError_t gi_bucket_scan(unsigned int *a, unsigned int m, unsigned int *sums, cudaStream_t s)
{
    if (m == 0 || m > 1024u * 8192u) return cudaErrorInvalidValue;
    const int sb = (int)((m + 1023) / 1024);
    gi::scan_blocks<<<sb, 1024, 0, s>>>(a, (int)m, sums);
    gi::scan_sums<<<1, 1024, 0, s>>>(sums, sb);
    gi::scan_add<<<sb, 1024, 0, s>>>(a, (int)m, sums);
    return cudaGetLastError();
}

cudaError_t gi_launch_contacts(const float4 *pos, const float4 *vel, const LaunchTable &tab,
                               long long bodies, int max_end, unsigned int *work,
                               long long *delta, int nsm, cudaStream_t s, cudaStream_t s_warp,
                               cudaEvent_t ev_grid)
{
    if (tab.nruns <= 0) return cudaSuccess;
    const unsigned int m = gi_grid_buckets(bodies);
    if (m > 1024u * 8192u) return cudaErrorInvalidValue;
    if (reinterpret_cast<uintptr_t>(work) & 15u) return cudaErrorInvalidValue;
    float4 *spos = reinterpret_cast<float4 *>(work);
    float4 *svel = spos + bodies;
    unsigned int *keys = work + 8 * (size_t)bodies;
    int *sorted = reinterpret_cast<int *>(keys + max_end);
    unsigned int *cursor = keys + 2 * (size_t)max_end;
    unsigned int *state = cursor + m;
    unsigned int *sums = state + m;
    unsigned int *ctr = sums + 8192;
    unsigned int *ntiled = ctr + gi::kCtrTiled;
    uint4 *raw = reinterpret_cast<uint4 *>((reinterpret_cast<uintptr_t>(ctr + gi::kCtrWords) + 15) &
                                           ~static_cast<uintptr_t>(15));
    const size_t icap = gi_dense_item_capacity(bodies);
    uint4 *items = raw + icap;
    unsigned int *tiled = reinterpret_cast<unsigned int *>(items + icap);
    int maxn = 0;
    for (int r = 0; r < tab.nruns; ++r) maxn = std::max(maxn, tab.runs[r].n);
    if (maxn == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(cursor, 0, (size_t)m * sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(state, 0, (size_t)m * sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(ctr, 0, gi::kCtrWords * sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    const dim3 gk(std::min(4 * nsm, (maxn + 255) / 256), tab.nruns);
    gi::grid_keys<<<gk, 256, 0, s>>>(pos, tab, m - 1, keys, cursor);
    const int sb = (int)((m + 1023) / 1024);
    gi::scan_blocks<<<sb, 1024, 0, s>>>(cursor, (int)m, sums);
    gi::scan_sums<<<1, 1024, 0, s>>>(sums, sb);
    gi::scan_add<<<sb, 1024, 0, s>>>(cursor, (int)m, sums);
    gi::grid_scatter<<<gk, 256, 0, s>>>(pos, vel, tab, keys, cursor, sorted, spos, svel);
    const unsigned int dmin = (unsigned int)tab.dense_min;
    gi::dense_check_kernel<<<gk, 256, 0, s>>>(pos, tab, keys, cursor, sorted, dmin, state, delta);
    gi::dense_mark_kernel<<<std::min((int)((m + 255) / 256), 4 * nsm), 256, 0, s>>>(
        pos, tab, cursor, sorted, m, m - 1, dmin, state, tiled, ntiled);
    gi::dense_sort_kernel<<<2 * nsm, 256, 0, s>>>(pos, vel, cursor, sorted, spos, svel, tiled, ntiled);
    const int gt = (int)std::min<size_t>((gi_dense_bucket_capacity(bodies) + 7) / 8, 4 * (size_t)nsm);
    gi::dense_items_kernel<<<gt, 256, 0, s>>>(pos, tab, cursor, sorted, m - 1, state, tiled, ctr,
                                              raw);
    const int go = (int)std::min<size_t>((icap + 255) / 256, 4 * (size_t)nsm);
    gi::dense_order_kernel<<<go, 256, 0, s>>>(raw, ctr, items);
    // The two contact kernels write disjoint bodies (the warp path skips
    // tiled buckets; the tiled path adds only into tiled bodies), so the
    // warp path may run on a stream of its own.  64-thread blocks (2
    // bodies): small enough to run beside the far field's CTAs in the
    // registers they leave free.
    cudaStream_t sw = s;
    if (s_warp && ev_grid) {
        e = cudaEventRecord(ev_grid, s);
        if (e != cudaSuccess) return e;
        e = cudaStreamWaitEvent(s_warp, ev_grid, 0);
        if (e != cudaSuccess) return e;
        sw = s_warp;
    }
    const dim3 gc((maxn + 1) / 2, tab.nruns);
    gi::contact_kernel<<<gc, 64, 0, sw>>>(pos, vel, spos, svel, cursor, sorted, keys, state,
                                          m - 1, delta, tab);
    gi::contact_tile_kernel<<<16 * nsm, 128, 0, s>>>(spos, svel, cursor, sorted, state, delta, tab,
                                                     items, ctr);
    return cudaGetLastError();
}
