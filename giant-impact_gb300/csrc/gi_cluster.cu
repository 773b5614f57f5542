// gi_cluster.cu -- Earth / Moon identification on the GPU.
//
// The reference (findEarthAndMoon, impactBasicFunctions.h:109-217) grows
// groups on the host by repeated O(N) scans: a body joins a group when its
// FP32 distance sqrtf(dx*dx + dy*dy + dz*dz) to a member is below
// touch = 1.5 D, and a group is numbered by the index of the body that
// started it, which is its smallest index.  Those groups are exactly the
// connected components of the "touching" graph, so here:
//
//   1. grid: cell = touch * (1 + 2^-10), computed in double, so two touching
//      bodies are always in the same or adjacent cells; cells hashed into
//      M = 2^k >= 2N buckets, counting sort (as the contact pass does);
//   2. union: one thread per body i visits the 27 neighbour buckets and, for
//      every j > i that touches i (the reference's FP32 test, evaluated with
//      the same roundings), links the two trees.  Links always hang the root
//      with the larger index under the one with the smaller index (one
//      atomicCAS on a root), so a tree's root is its smallest member: the
//      reference's group number;
//   3. flatten: group[i] = root of i (found without writes, so that no
//      thread overwrites a final root); sizes by atomicAdd;
//   4. pick: Earth = largest group, smallest name on a tie (the reference's
//      first strict maximum); Moon = largest of the others; both by a 64-bit
//      atomicMax of (size << 32 | ~name);
//   5. tag: scope byte (1 Earth, 2 Moon) and the origin counts.
// Every loop is bounded: a failed link moves to a strictly smaller index, so
// a link takes at most N tries; the kernels still stop after a set number
// (gi_options.cluster_tries, 2^22 by default) and raise an error flag that
// the host turns into GI_ERR_TIMEOUT.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "gi_internal.h"

namespace gi {

__device__ __forceinline__ int cluster_cell(float x, double inv_cell)
{
    double f = floor((double)x * inv_cell);
    if (!(f >= -1.0e9)) f = -1.0e9;  // also NaN
    if (f > 1.0e9) f = 1.0e9;
    return (int)f;
}

__device__ __forceinline__ unsigned int cluster_bucket(int cx, int cy, int cz, unsigned int mask)
{
    unsigned int h = (unsigned int)cx * 2246822519u;
    h ^= (unsigned int)cy * 3266489917u;
    h ^= (unsigned int)cz * 668265263u;
    h ^= h >> 13;
    h *= 2654435761u;
    h ^= h >> 16;
    return h & mask;
}

__global__ void __launch_bounds__(256)
cluster_keys(const float4 *__restrict__ pos, int n, double inv_cell, unsigned int mask,
             unsigned int *__restrict__ keys, unsigned int *__restrict__ hist,
             int *__restrict__ parent)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = pos[i];
        const unsigned int b = cluster_bucket(cluster_cell(p.x, inv_cell), cluster_cell(p.y, inv_cell),
                                              cluster_cell(p.z, inv_cell), mask);
        keys[i] = b;
        parent[i] = i;
        atomicAdd(&hist[b], 1u);
    }
}

__global__ void __launch_bounds__(256)
cluster_scatter(int n, const unsigned int *__restrict__ keys, unsigned int *__restrict__ cursor,
                int *__restrict__ sorted)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned int slot = atomicAdd(&cursor[keys[i]], 1u);
        sorted[slot] = i;
    }
}

// Root of x with path halving.  Every parent pointer points to an ancestor
// with a smaller index, so x strictly decreases and the loop ends.
__device__ __forceinline__ int find_root(int *parent, int x)
{
    for (;;) {
        const int p = __ldcg(&parent[x]);
        if (p == x) return x;
        const int g = __ldcg(&parent[p]);
        if (g == p) return p;
        __stcg(&parent[x], g);
        x = g;
    }
}

// Root of x without writes.  The flatten pass writes every body's final
// root; a path-halving write from another thread, based on a parent read
// before that write, could replace it with an intermediate ancestor.
__device__ __forceinline__ int find_root_ro(const int *parent, int x)
{
    for (;;) {
        const int p = __ldcg(&parent[x]);
        if (p == x) return x;
        x = p;
    }
}

__device__ __forceinline__ bool link(int *parent, int a, int b, int tries)
{
    for (int t = 0; t < tries; ++t) {
        a = find_root(parent, a);
        b = find_root(parent, b);
        if (a == b) return true;
        if (a < b) { const int s = a; a = b; b = s; }
        const int old = atomicCAS(&parent[a], a, b);
        if (old == a) return true;
        a = old;
    }
    return false;
}

// The reference's touch test: sqrtf of ((dx*dx + dy*dy) + dz*dz), each
// operation rounded separately (host code without contraction).
__device__ __forceinline__ bool touching(float4 a, float4 b, float touch)
{
    const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
    const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    return __fsqrt_rn(r2) < touch;
}

__global__ void __launch_bounds__(256)
cluster_union(const float4 *__restrict__ pos, int n, const unsigned int *__restrict__ cursor,
              const int *__restrict__ sorted, unsigned int mask, double inv_cell, float touch,
              int tries, int *parent, int *__restrict__ err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 pi = pos[i];
    const int cx = cluster_cell(pi.x, inv_cell), cy = cluster_cell(pi.y, inv_cell),
              cz = cluster_cell(pi.z, inv_cell);
    unsigned int seen[27];
    int nseen = 0;
    for (int o = 0; o < 27; ++o) {
        const unsigned int b =
            cluster_bucket(cx + o % 3 - 1, cy + (o / 3) % 3 - 1, cz + o / 9 - 1, mask);
        bool dup = false;
        for (int q = 0; q < nseen; ++q) dup |= seen[q] == b;
        if (dup) continue;
        seen[nseen++] = b;
        const unsigned int beg = b ? cursor[b - 1] : 0u, end = cursor[b];
        for (unsigned int s = beg; s < end; ++s) {
            const int j = sorted[s];
            if (j <= i) continue;
            if (!touching(pi, pos[j], touch)) continue;
            if (!link(parent, i, j, tries)) atomicExch(err, 1);
        }
    }
}

__global__ void __launch_bounds__(256)
cluster_flatten(int *parent, int n, int *__restrict__ size, int *__restrict__ ngroups)
{
    int roots = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int r = find_root_ro(parent, i);
        __stcg(&parent[i], r);
        atomicAdd(&size[r], 1);
        roots += r == i;
    }
    for (int o = 16; o > 0; o >>= 1) roots += __shfl_down_sync(0xffffffffu, roots, o);
    if ((threadIdx.x & 31) == 0 && roots) atomicAdd(ngroups, roots);
}

__device__ __forceinline__ unsigned long long group_key(int size, int name)
{
    return ((unsigned long long)(unsigned int)size << 32) | (unsigned int)(~(unsigned int)name);
}

__device__ __forceinline__ int key_name(unsigned long long k)
{
    return k ? (int)(~(unsigned int)(k & 0xffffffffull)) : -1;
}

// exclude_key: the Earth's key when picking the Moon, NULL when picking the Earth.
__global__ void __launch_bounds__(256)
cluster_pick(const int *__restrict__ group, const int *__restrict__ size, int n,
             const unsigned long long *exclude_key, unsigned long long *best)
{
    const int skip = exclude_key ? key_name(*exclude_key) : -1;
    unsigned long long k = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (group[i] == i && i != skip) k = max(k, group_key(size[i], i));
    for (int o = 16; o > 0; o >>= 1) k = max(k, __shfl_down_sync(0xffffffffu, k, o));
    if ((threadIdx.x & 31) == 0 && k) atomicMax(best, k);
}

// keys[0] Earth, keys[1] Moon; counts[0..3] Earth, [4..7] Moon by origin.
__global__ void __launch_bounds__(256)
cluster_tag(const int *__restrict__ group, int n, const unsigned long long *__restrict__ keys,
            int b0, int b1, int b2, int *__restrict__ group_out,
            unsigned char *__restrict__ scope_out, int *__restrict__ counts)
{
    __shared__ int sc[8];
    if (threadIdx.x < 8) sc[threadIdx.x] = 0;
    __syncthreads();
    const int earth = key_name(keys[0]), moon = key_name(keys[1]);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int g = group[i];
        const unsigned char s = g == earth ? 1 : (g == moon ? 2 : 0);
        if (group_out) group_out[i] = g;
        if (scope_out) scope_out[i] = s;
        if (s) {
            const int c = i < b0 ? 0 : (i < b1 ? 1 : (i < b2 ? 2 : 3));
            atomicAdd(&sc[4 * (s - 1) + c], 1);
        }
    }
    __syncthreads();
    if (threadIdx.x < 8 && sc[threadIdx.x]) atomicAdd(&counts[threadIdx.x], sc[threadIdx.x]);
}

}  // namespace gi

namespace {

struct ClusterResult {
    unsigned long long keys[2];
    int counts[8];
    int ngroups;
    int err;
};

int cuda_status(cudaError_t e, const char *what)
{
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    return gi_internal_fail(e == cudaErrorMemoryAllocation ? GI_ERR_OUT_OF_MEMORY : GI_ERR_CUDA, buf);
}

}  // namespace

extern "C" int gi_find_earth_moon(gi_ctx *ctx, const float *pos, int n, float touch,
                                  const int bounds[3], int *group, unsigned char *scope,
                                  gi_earth_moon *out, void *stream)
{
    if (!ctx || !out || !bounds || (n > 0 && !pos) || n < 0)
        return gi_internal_fail(GI_ERR_INVALID_ARG, "gi_find_earth_moon: NULL argument or n < 0");
    if (!(touch > 0.0f) || !(touch < 1.0e30f))
        return gi_internal_fail(GI_ERR_INVALID_ARG, "gi_find_earth_moon: touch must be positive");
    if (reinterpret_cast<uintptr_t>(pos) % 16)
        return gi_internal_fail(GI_ERR_ALIGNMENT, "gi_find_earth_moon: pos not 16-byte aligned");
    std::memset(out, 0, sizeof *out);
    out->earth_label = out->moon_label = -1;
    if (n == 0) return GI_OK;
    const int dev = gi_internal_ctx_device(ctx);
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
    struct Restore {
        int prev, dev;
        ~Restore()
        {
            if (prev != dev && prev >= 0) cudaSetDevice(prev);
        }
    } restore{prev, dev};
    cudaStream_t s = (cudaStream_t)stream;
    unsigned int m = 1024;
    while (m < 2u * (unsigned int)n && m < (1u << 30)) m <<= 1;
    if (m > 1024u * 8192u) return gi_internal_fail(GI_ERR_BAD_SIZE, "gi_find_earth_moon: n too large");
    // one allocation: parent, size, keys, sorted (n each), cursor (m),
    // scan sums (8192), result
    const size_t words = 4 * (size_t)n + m + 8192;
    const size_t bytes = words * 4 + sizeof(ClusterResult) + 16;
    unsigned char *buf = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, bytes, s);
    if (e != cudaSuccess) return cuda_status(e, "cudaMallocAsync");
    int *parent = reinterpret_cast<int *>(buf);
    int *size = parent + n;
    unsigned int *keys = reinterpret_cast<unsigned int *>(size + n);
    int *sorted = reinterpret_cast<int *>(keys + n);
    unsigned int *cursor = reinterpret_cast<unsigned int *>(sorted + n);
    unsigned int *sums = cursor + m;
    size_t roff = (words * 4 + 15) & ~(size_t)15;
    ClusterResult *res = reinterpret_cast<ClusterResult *>(buf + roff);
    ClusterResult host{};
    const double inv_cell = 1.0 / ((double)touch * (1.0 + 1.0 / 1024.0));
    const int blocks = (n + 255) / 256;
    const int gridded = std::min(blocks, 4096);
    do {
        if ((e = cudaMemsetAsync(size, 0, (size_t)n * 4, s)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(cursor, 0, (size_t)m * 4, s)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(res, 0, sizeof(ClusterResult), s)) != cudaSuccess) break;
        gi::cluster_keys<<<gridded, 256, 0, s>>>(reinterpret_cast<const float4 *>(pos), n, inv_cell,
                                                 m - 1, keys, cursor, parent);
        if ((e = gi_bucket_scan(cursor, m, sums, s)) != cudaSuccess) break;
        gi::cluster_scatter<<<gridded, 256, 0, s>>>(n, keys, cursor, sorted);
        // cursor[b] is now the end of bucket b
        gi::cluster_union<<<blocks, 256, 0, s>>>(reinterpret_cast<const float4 *>(pos), n, cursor,
                                                 sorted, m - 1, inv_cell, touch,
                                                 gi_internal_ctx_cluster_tries(ctx), parent,
                                                 &res->err);
        gi::cluster_flatten<<<gridded, 256, 0, s>>>(parent, n, size, &res->ngroups);
        gi::cluster_pick<<<gridded, 256, 0, s>>>(parent, size, n, nullptr, &res->keys[0]);
        gi::cluster_pick<<<gridded, 256, 0, s>>>(parent, size, n, &res->keys[0], &res->keys[1]);
        gi::cluster_tag<<<gridded, 256, 0, s>>>(parent, n, res->keys, bounds[0], bounds[1],
                                                bounds[2], group, scope, res->counts);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(&host, res, sizeof host, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            break;
    } while (false);
    const cudaError_t ef = cudaFreeAsync(buf, s);
    if (e == cudaSuccess) e = ef;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "gi_find_earth_moon");
    if (host.err) return gi_internal_fail(GI_ERR_TIMEOUT, "gi_find_earth_moon: a link did not settle");
    auto name = [](unsigned long long k) { return k ? (int)(~(unsigned int)(k & 0xffffffffull)) : -1; };
    out->earth_label = name(host.keys[0]);
    out->moon_label = name(host.keys[1]);
    out->n_earth = (int)(host.keys[0] >> 32);
    out->n_moon = (int)(host.keys[1] >> 32);
    out->n_groups = host.ngroups;
    for (int c = 0; c < 4; ++c) {
        out->earth_counts[c] = host.counts[c];
        out->moon_counts[c] = host.counts[4 + c];
    }
    return GI_OK;
}

// ------------------------------------------------------------------ disk --

namespace gi {

// Largest distance of an Earth element (scope 1) from the Earth's centre of
// mass, as the bits of a non-negative double (ordered like the value).
__global__ void __launch_bounds__(256)
earth_radius_kernel(const float4 *__restrict__ pos, const unsigned char *__restrict__ scope, int off,
                    int n, double cx, double cy, double cz, unsigned long long *__restrict__ rmax)
{
    double m = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = off + k;
        if (scope[i] != 1) continue;
        const float4 p = pos[i];
        const double dx = p.x - cx, dy = p.y - cy, dz = p.z - cz;
        m = fmax(m, sqrt(dx * dx + dy * dy + dz * dz));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(rmax, (unsigned long long)__double_as_longlong(m));
}

// counts: [disk, bound inside, unbound]
__global__ void __launch_bounds__(256)
disk_kernel(const float4 *__restrict__ pos, const float4 *__restrict__ vel,
            unsigned char *__restrict__ scope, int off, int n, double cx, double cy, double cz,
            double ux, double uy, double uz, double gm, const unsigned long long *__restrict__ rmax,
            int *__restrict__ counts)
{
    __shared__ int sc[3];
    if (threadIdx.x < 3) sc[threadIdx.x] = 0;
    __syncthreads();
    const double R = __longlong_as_double((long long)*rmax) + 0.5;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = off + k;
        const unsigned char s = scope[i];
        if (s == 1 || s == 2) continue;
        const float4 p = pos[i], u = vel[i];
        const double rx = p.x - cx, ry = p.y - cy, rz = p.z - cz;
        const double vx = u.x - ux, vy = u.y - uy, vz = u.z - uz;
        const double r = sqrt(rx * rx + ry * ry + rz * rz);
        const double eps = 0.5 * (vx * vx + vy * vy + vz * vz) - gm / r;
        const double hx = ry * vz - rz * vy, hy = rz * vx - rx * vz, hz = rx * vy - ry * vx;
        const double req = (hx * hx + hy * hy + hz * hz) / gm;
        int c;
        if (eps < 0.0) c = req > R ? 0 : 1;
        else c = 2;
        scope[i] = c == 0 ? 3 : 0;
        atomicAdd(&sc[c], 1);
    }
    __syncthreads();
    if (threadIdx.x < 3 && sc[threadIdx.x]) atomicAdd(&counts[threadIdx.x], sc[threadIdx.x]);
}

}  // namespace gi

extern "C" int gi_find_disk(gi_ctx *ctx, const float *pos, const float *vel, const gi_run *run,
                            const gi_pair_params *params, unsigned char *scope, gi_disk_info *out,
                            void *stream)
{
    if (!ctx || !pos || !vel || !run || !params || !scope || !out)
        return gi_internal_fail(GI_ERR_INVALID_ARG, "gi_find_disk: NULL argument");
    if (run->n < 0 || run->offset < 0)
        return gi_internal_fail(GI_ERR_BAD_SIZE, "gi_find_disk: bad run");
    if (!(params->MassSi > 0.0f) || !(params->GMassSiSi > 0.0f))
        return gi_internal_fail(GI_ERR_PARAMS, "gi_find_disk: masses and gravity must be positive");
    std::memset(out, 0, sizeof *out);
    double earth[15];
    if (int st = gi_diag_fp64(ctx, pos, vel, scope, 2, run, params, earth, stream)) return st;
    out->earth_mass = earth[0];
    if (run->n == 0 || !(earth[0] > 0.0)) return GI_OK;  // no Earth: nothing is bound to it
    const double G = (double)params->GMassSiSi / ((double)params->MassSi * params->MassSi);
    const int dev = gi_internal_ctx_device(ctx);
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
    struct Restore {
        int prev, dev;
        ~Restore()
        {
            if (prev != dev && prev >= 0) cudaSetDevice(prev);
        }
    } restore{prev, dev};
    cudaStream_t s = (cudaStream_t)stream;
    struct Res {
        unsigned long long rmax;
        int counts[3];
        int pad;
    };
    Res *res = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&res), sizeof(Res), s);
    if (e != cudaSuccess) return cuda_status(e, "cudaMallocAsync");
    Res host{};
    const int blocks = std::min((run->n + 255) / 256, 4096);
    const float4 *P = reinterpret_cast<const float4 *>(pos);
    do {
        if ((e = cudaMemsetAsync(res, 0, sizeof(Res), s)) != cudaSuccess) break;
        gi::earth_radius_kernel<<<blocks, 256, 0, s>>>(P, scope, run->offset, run->n, earth[1], earth[2],
                                                       earth[3], &res->rmax);
        gi::disk_kernel<<<blocks, 256, 0, s>>>(P, reinterpret_cast<const float4 *>(vel), scope,
                                               run->offset, run->n, earth[1], earth[2], earth[3],
                                               earth[4], earth[5], earth[6], G * earth[0], &res->rmax,
                                               res->counts);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(&host, res, sizeof host, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            break;
    } while (false);
    const cudaError_t ef = cudaFreeAsync(res, s);
    if (e == cudaSuccess) e = ef;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "gi_find_disk");
    double r = 0.0;
    std::memcpy(&r, &host.rmax, sizeof r);
    out->earth_radius = r + 0.5;
    out->n_disk = host.counts[0];
    out->n_bound_inside = host.counts[1];
    out->n_unbound = host.counts[2];
    return GI_OK;
}
