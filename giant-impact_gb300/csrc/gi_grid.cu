// gi_grid.cu -- contact forces through a hashed cell grid.
//
// The all-pairs kernel evaluates far-field gravity for every pair with r2
// clamped at one diameter.  The pairs inside one diameter (r2 < 1, the only
// ones where the reference law departs from gravity) are handled here:
//
//   1. grid: every body gets the cell floor(x), floor(y), floor(z) (cell size
//      D = 1, so two bodies within r < 1 are in the same or adjacent cells),
//      hashed with its run into M = 2^k buckets; a counting sort (histogram,
//      exclusive scan, scatter) lists the bodies of each bucket.
//   2. contact kernel: one warp per body scans the buckets of its 27
//      neighbour cells; for each j of the same run with FP32 r2 < 1 it adds
//          contact force of the reference law  -  the clamped far-field term
//      the all-pairs pass added for that pair.  Band and K/KR choices use the
//      reference's FP32 r2 and dp.dv (bit-identical decisions).
//   3. each pair's correction is evaluated in FP32 and summed in 64-bit
//      fixed point (unit = (2 Gmax + Kmax) 2^-40 per pair table): integer
//      adds are exact, so the sum does not depend on the order in which
//      bodies landed in buckets or lanes found them, and the result is
//      bit-reproducible.
// The all-pairs epilogue adds the correction before its single rounding.
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

// After this, bucket b holds sorted[(b ? cursor[b-1] : 0) .. cursor[b]).
__global__ void __launch_bounds__(256)
grid_scatter(const __grid_constant__ LaunchTable tab, const unsigned int *__restrict__ keys,
             unsigned int *__restrict__ cursor, int *__restrict__ sorted)
{
    const RunDev &R = tab.runs[blockIdx.y];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < R.n; k += gridDim.x * blockDim.x) {
        const int i = R.offset + k;
        const unsigned int slot = atomicAdd(&cursor[keys[i]], 1u);
        sorted[slot] = i;
    }
}

// Contact correction of one pair, as a coefficient of dp in force units:
// the reference law's contact force on i, mag dp / r, minus the clamped
// far-field term gm_i gm_j r2c^-3/2 dp the all-pairs pass added.
__device__ __forceinline__ float contact_coef(const PairDev &P, int sep_test, int i, int j,
                                              int sw, float dx, float dy, float dz, float r2,
                                              float4 vi, float4 vj)
{
    const int test = (i < sw) + (j < sw);
    const float G = P.G[test];
    float K = P.K[test];
    if (!(r2 >= P.Tband[test])) {
        const float dvx = __fsub_rn(vj.x, vi.x), dvy = __fsub_rn(vj.y, vi.y),
                    dvz = __fsub_rn(vj.z, vi.z);
        const float dpdv = __fmaf_rn(dz, dvz, __fmaf_rn(dx, dvx, __fmul_rn(dy, dvy)));
        // Reference: int inout = dp.dv; KR when inout > 0, i.e. dp.dv >= 1.
        const bool sep = (sep_test == GI_SEP_SIGN) ? (dpdv > 0.0f) : (dpdv >= 1.0f);
        if (sep) K = (r2 >= P.Tmid[test]) ? P.KRmid[test] : P.KRin[test];
    }
    const float mag = contact_mag(G, K, r2);
    const float invr = __fdiv_rn(1.0f, __fsqrt_rn(r2));
    const float ri = rsqrt_mufu(fmaxf(r2, 1.0f));
    const float s_far = (ri * ri) * ri;
    const float gmi = (i < sw) ? P.gm_fe : P.gm_si;
    const float gmj = (j < sw) ? P.gm_fe : P.gm_si;
    return __fmaf_rn(mag, invr, -(gmi * gmj) * s_far);
}

// One warp per body.  Lanes 0..26 look up the 27 neighbour buckets at once
// (one memory round trip; a bucket that two neighbour cells share is kept
// once), a warp scan lays their bodies end to end, and the warp then walks
// that list 32 candidates at a time.
__global__ void __launch_bounds__(256)
contact_kernel(const float4 *__restrict__ pos, const float4 *__restrict__ vel,
               const unsigned int *__restrict__ cursor, const int *__restrict__ sorted,
               unsigned int mask, long long *__restrict__ delta,
               const __grid_constant__ LaunchTable tab)
{
    const RunDev &R = tab.runs[blockIdx.y];
    const PairDev &P = tab.params[R.param];
    const int lane = threadIdx.x & 31;
    const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k >= R.n) return;  // whole warp leaves together
    const int i = R.offset + k;
    const int rbeg = R.offset, rend = R.offset + R.n, sw = R.offset + R.nfe;
    const float4 pi = __ldg(&pos[i]);
    const int cx = cell_of(pi.x), cy = cell_of(pi.y), cz = cell_of(pi.z);

    unsigned int b = 0xffffffffu, beg = 0u, cnt = 0u;
    if (lane < 27) {
        const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
        b = bucket_of(blockIdx.y, cx + ox, cy + oy, cz + oz, mask);
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

    const float inv_unit = (float)(1.0 / P.fx_unit);
    float4 vi = make_float4(0.f, 0.f, 0.f, 0.f);
    bool have_vi = false;
    long long ax = 0, ay = 0, az = 0;
    for (unsigned int base = 0; base < total; base += 32) {
        const unsigned int t = base + lane;
        // the lane whose range [excl, incl) holds t: last lane with excl <= t
        int src = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const unsigned int e = __shfl_sync(0xffffffffu, excl, src + step);
            if (src + step < 32 && e <= t) src += step;
        }
        const unsigned int sb = __shfl_sync(0xffffffffu, beg, src);
        const unsigned int se = __shfl_sync(0xffffffffu, excl, src);
        if (t >= total) continue;
        const int j = __ldg(&sorted[sb + (t - se)]);
        if (j == i || j < rbeg || j >= rend) continue;
        const float4 pj = __ldg(&pos[j]);
        const float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
        if (!(r2 < 1.0f)) continue;
        if (!have_vi) { vi = __ldg(&vel[i]); have_vi = true; }
        const float4 vj = __ldg(&vel[j]);
        const float c = contact_coef(P, tab.sep_test, i, j, sw, dx, dy, dz, r2, vi, vj) * inv_unit;
        ax += __float2ll_rn(c * dx);
        ay += __float2ll_rn(c * dy);
        az += __float2ll_rn(c * dz);
    }
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

}  // namespace gi

// Buckets of the grid for `bodies` bodies: a power of two >= 2 * bodies.
unsigned int gi_grid_buckets(long long bodies)
{
    unsigned long long m = 1024;
    while (m < 2ull * (unsigned long long)bodies) m <<= 1;
    return (unsigned int)m;
}

// keys + sorted: `bodies` each (indexed by global body index / slot); cursor:
// buckets; block sums: 8192.
size_t gi_grid_words(long long max_end, long long bodies)
{
    return 2 * (size_t)max_end + gi_grid_buckets(bodies) + 8192;
}

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
                               long long *delta, int nsm, cudaStream_t s)
{
    if (tab.nruns <= 0) return cudaSuccess;
    const unsigned int m = gi_grid_buckets(bodies);
    if (m > 1024u * 8192u) return cudaErrorInvalidValue;
    unsigned int *keys = work;
    int *sorted = reinterpret_cast<int *>(work + max_end);
    unsigned int *cursor = work + 2 * (size_t)max_end;
    unsigned int *sums = cursor + m;
    int maxn = 0;
    for (int r = 0; r < tab.nruns; ++r) maxn = std::max(maxn, tab.runs[r].n);
    if (maxn == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(cursor, 0, (size_t)m * sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    const dim3 gk(std::min(4 * nsm, (maxn + 255) / 256), tab.nruns);
    gi::grid_keys<<<gk, 256, 0, s>>>(pos, tab, m - 1, keys, cursor);
    const int sb = (int)((m + 1023) / 1024);
    gi::scan_blocks<<<sb, 1024, 0, s>>>(cursor, (int)m, sums);
    gi::scan_sums<<<1, 1024, 0, s>>>(sums, sb);
    gi::scan_add<<<sb, 1024, 0, s>>>(cursor, (int)m, sums);
    gi::grid_scatter<<<gk, 256, 0, s>>>(tab, keys, cursor, sorted);
    const dim3 gc((maxn + 7) / 8, tab.nruns);
    gi::contact_kernel<<<gc, 256, 0, s>>>(pos, vel, cursor, sorted, m - 1, delta, tab);
    return cudaGetLastError();
}
