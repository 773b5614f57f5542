// gi_api.cu -- the C ABI of libgi.so: argument checking, the work-decomposition
// planner, context-owned scratch memory and the entry points declared in
// include/gi_api.h.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "gi_internal.h"

int gi_force_occupancy_ipt1(int acc, int epi);
int gi_force_occupancy_ipt2(int acc, int epi);
int gi_force_occupancy_ipt4(int acc, int epi);
int gi_force_occupancy_ipt8(int acc, int epi);

// ------------------------------------------------------------------ errors --

static thread_local std::string g_last_error;

static int fail(int status, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

static int cuda_fail(cudaError_t e, const char *what)
{
    int st = (e == cudaErrorMemoryAllocation) ? GI_ERR_OUT_OF_MEMORY
             : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ||
                e == cudaErrorNoKernelImageForDevice)
                 ? GI_ERR_NO_DEVICE
                 : GI_ERR_CUDA;
    return fail(st, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

#define GI_CUDA(call, what)                                \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

extern "C" int gi_version(void) { return GI_API_VERSION; }

extern "C" const char *gi_status_string(int s)
{
    switch (s) {
    case GI_OK: return "ok";
    case GI_ERR_INVALID_ARG: return "invalid argument";
    case GI_ERR_BAD_SIZE: return "size out of range";
    case GI_ERR_ALIGNMENT: return "body array not 16-byte aligned";
    case GI_ERR_CUDA: return "CUDA error";
    case GI_ERR_TIMEOUT: return "device wait timed out";
    case GI_ERR_NO_DEVICE: return "no usable CUDA device";
    case GI_ERR_OUT_OF_MEMORY: return "out of device memory";
    case GI_ERR_PARAMS: return "inconsistent physical parameters";
    case GI_ERR_IO: return "file I/O error";
    case GI_ERR_FORMAT: return "malformed file";
    case GI_ERR_CAPACITY: return "capacity exceeded";
    default: return "unknown status";
    }
}

extern "C" const char *gi_last_error(void) { return g_last_error.c_str(); }

extern "C" int gi_device_info(int device, int *sm_count, int *cc_major, int *cc_minor,
                              long long *global_mem_bytes)
{
    cudaDeviceProp prop;
    GI_CUDA(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    if (sm_count) *sm_count = prop.multiProcessorCount;
    if (cc_major) *cc_major = prop.major;
    if (cc_minor) *cc_minor = prop.minor;
    if (global_mem_bytes) *global_mem_bytes = (long long)prop.totalGlobalMem;
    return GI_OK;
}

cudaError_t gi_launch_force(int ipt, int acc, int epi, const ForceArgs &a,
                            const LaunchTable &tab, int grid, cudaStream_t s)
{
    switch (ipt) {
    case 1: return gi_launch_force_ipt1(acc, epi, a, tab, grid, s);
    case 2: return gi_launch_force_ipt2(acc, epi, a, tab, grid, s);
    case 4: return gi_launch_force_ipt4(acc, epi, a, tab, grid, s);
    case 8: return gi_launch_force_ipt8(acc, epi, a, tab, grid, s);
    default: return cudaErrorInvalidValue;
    }
}

int gi_force_occupancy(int ipt, int acc, int epi)
{
    switch (ipt) {
    case 1: return gi_force_occupancy_ipt1(acc, epi);
    case 2: return gi_force_occupancy_ipt2(acc, epi);
    case 4: return gi_force_occupancy_ipt4(acc, epi);
    case 8: return gi_force_occupancy_ipt8(acc, epi);
    default: return 0;
    }
}

// ------------------------------------------------------------- parameters --

// Smallest float t with sqrtf(t) >= s: the reference's "s <= sqrt(r2)"
// band test (impactAddTime.cu:304, 324, 328, 353) becomes "r2 >= t".
static float r2_threshold(float s)
{
    if (!(s > 0.0f)) return 0.0f;
    float t = s * s;
    while (sqrtf(t) < s) t = nextafterf(t, INFINITY);
    while (t > 0.0f && sqrtf(nextafterf(t, -INFINITY)) >= s) t = nextafterf(t, -INFINITY);
    return t;
}

static int to_device_params(const gi_pair_params &p, PairDev &d)
{
    const float vals[] = {p.GMassFeFe, p.GMassFeSi, p.GMassSiSi, p.KFeFe, p.KSiSi, p.KFeSi,
                          p.KRFeFe, p.KRSiSi, p.KRFeSi, p.KRMix, p.ShellBreakFe,
                          p.ShellBreakSi, p.ShellBreakFeSi1, p.ShellBreakFeSi2};
    for (float v : vals)
        if (!std::isfinite(v)) return fail(GI_ERR_PARAMS, "pair table holds a non-finite value");
    if (!(p.GMassFeFe > 0.0f) || !(p.GMassSiSi > 0.0f) || !(p.GMassFeSi > 0.0f))
        return fail(GI_ERR_PARAMS, "G*m*m must be positive for every pair class");
    // The far-field loop factorises G m_i m_j = gm_i gm_j.
    const double gfe = std::sqrt((double)p.GMassFeFe), gsi = std::sqrt((double)p.GMassSiSi);
    const double cross = gfe * gsi, want = (double)p.GMassFeSi;
    if (std::fabs(cross - want) > 1e-5 * std::max(std::fabs(want), 1e-30) + 1e-30)
        return fail(GI_ERR_PARAMS,
                    "gravity table is not rank one: GMassFeSi^2 (%g) != GMassFeFe*GMassSiSi (%g)",
                    want * want, (double)p.GMassFeFe * p.GMassSiSi);
    d.gm_fe = (float)gfe;
    d.gm_si = (float)gsi;
    d.G[0] = p.GMassSiSi; d.G[1] = p.GMassFeSi; d.G[2] = p.GMassFeFe;
    d.K[0] = p.KSiSi; d.K[1] = p.KFeSi; d.K[2] = p.KFeFe;
    d.KRmid[0] = p.KRSiSi; d.KRmid[1] = p.KRMix; d.KRmid[2] = p.KRFeFe;
    d.KRin[0] = p.KRSiSi; d.KRin[1] = p.KRFeSi; d.KRin[2] = p.KRFeFe;
    d.Tband[0] = r2_threshold(p.ShellBreakSi);
    d.Tband[1] = r2_threshold(p.ShellBreakFeSi1);
    d.Tband[2] = r2_threshold(p.ShellBreakFe);
    d.Tmid[0] = d.Tband[0];
    d.Tmid[1] = r2_threshold(p.ShellBreakFeSi2);
    d.Tmid[2] = d.Tband[2];
    // Contact corrections are summed in 64-bit fixed point: one pair's
    // correction is at most |G - K (1 - r2)| + G m m <= 2 Gmax + Kmax, which
    // maps to 2^40 units, leaving room for 2^22 contacts per body.
    double gmax = 0.0, kmax = 0.0;
    for (int t = 0; t < 3; ++t) {
        gmax = std::max(gmax, (double)std::fabs(d.G[t]));
        kmax = std::max({kmax, (double)std::fabs(d.K[t]), (double)std::fabs(d.KRmid[t]),
                         (double)std::fabs(d.KRin[t])});
    }
    d.fx_unit = std::ldexp(2.0 * gmax + kmax, -40);
    d.inv_unit = (float)(1.0 / d.fx_unit);
    return GI_OK;
}

extern "C" int gi_params_from_material(double G, double D, double mfe, double msi,
                                       double kfe, double ksi, double krfe, double krsi,
                                       double sdfe, double sdsi, gi_pair_params *o)
{
    if (!o) return fail(GI_ERR_INVALID_ARG, "out is NULL");
    // impactAddTime.cu:128-170 / generateTargetImpactor.cu:406-451, computed
    // in double and stored as float like the reference structs.
    o->GMassFeFe = (float)(G * mfe * mfe);
    o->GMassFeSi = (float)(G * mfe * msi);
    o->GMassSiSi = (float)(G * msi * msi);
    o->KFeFe = (float)(2.0 * kfe);
    o->KSiSi = (float)(2.0 * ksi);
    o->KFeSi = (float)(kfe + ksi);
    o->KRFeFe = (float)(2.0 * kfe * krfe);
    o->KRSiSi = (float)(2.0 * ksi * krsi);
    o->KRFeSi = (float)(kfe * krfe + ksi * krsi);
    o->KRMix = (float)((sdfe >= sdsi) ? kfe + ksi * krsi : kfe * krfe + ksi);
    o->ShellBreakFe = (float)(D - D * sdfe);
    o->ShellBreakSi = (float)(D - D * sdsi);
    if (sdfe >= sdsi) {
        o->ShellBreakFeSi1 = (float)(D - D * sdsi);
        o->ShellBreakFeSi2 = (float)(D - D * sdfe);
    } else {
        o->ShellBreakFeSi1 = (float)(D - D * sdfe);
        o->ShellBreakFeSi2 = (float)(D - D * sdsi);
    }
    o->MassFe = (float)mfe;
    o->MassSi = (float)msi;
    return GI_OK;
}

extern "C" int gi_params_from_collision_consts(const gi_force_collision_consts *c,
                                               gi_pair_params *o)
{
    if (!c || !o) return fail(GI_ERR_INVALID_ARG, "NULL argument");
    o->GMassFeFe = c->GMassFeFe;
    o->GMassFeSi = c->GMassFeSi;
    o->GMassSiSi = 1.0f;  // impactAddTime.cu:302: G = 1 and m_Si = 1
    o->KFeFe = c->KFeFe; o->KSiSi = c->KSiSi; o->KFeSi = c->KFeSi;
    o->KRFeFe = c->KRFeFe; o->KRSiSi = c->KRSiSi; o->KRFeSi = c->KRFeSi; o->KRMix = c->KRMix;
    o->ShellBreakFe = c->ShellBreakFe; o->ShellBreakSi = c->ShellBreakSi;
    o->ShellBreakFeSi1 = c->ShellBreakFeSi1; o->ShellBreakFeSi2 = c->ShellBreakFeSi2;
    o->MassFe = c->GMassFeSi;  // G = 1, m_Si = 1  =>  GMassFeSi = m_Fe
    o->MassSi = 1.0f;
    return GI_OK;
}

static void separate_params(const gi_force_separate_consts *c, gi_pair_params *o)
{
    gi_force_collision_consts cc;
    std::memcpy(&cc, c, offsetof(gi_force_collision_consts, NFe));
    cc.NFe = 0;
    gi_params_from_collision_consts(&cc, o);
}

// ---------------------------------------------------------------- context --

struct DeviceGuard {
    int prev = -1;
    bool changed = false;
    explicit DeviceGuard(int d)
    {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != d) {
            changed = cudaSetDevice(d) == cudaSuccess;
        }
    }
    ~DeviceGuard()
    {
        if (changed) cudaSetDevice(prev);
    }
};

// Scratch owned per stream, so that launches on different streams of one
// context never share a work queue, tickets or partial sums.
struct StreamScratch {
    // One allocation of counters: [0..1] the persistent kernel's work queue,
    // then one split ticket per i-block.  All of them are cleared on the
    // stream before every far-field launch, so a launch that was cut short
    // (an aborted kernel, a capture torn down) cannot leave the next one a
    // queue that skips work.
    unsigned int *counters = nullptr;
    unsigned int *queue = nullptr;    // counters + 0
    unsigned int *tickets = nullptr;  // counters + 2
    size_t tickets_cap = 0;
    double *partials = nullptr;       // split-j partial sums
    size_t partials_cap = 0;          // doubles
    float4 *pp_pos = nullptr, *pp_vel = nullptr;  // second state buffer of gi_step
    size_t pp_cap = 0;                // bodies
    unsigned int *grid_work = nullptr;  // cell grid of the contact pass (gi_grid.cu)
    size_t grid_work_cap = 0;           // words
    long long *delta = nullptr;         // contact corrections, 3 per body
    size_t delta_cap = 0;               // bodies
    double *fsum = nullptr;  // far-field sums, 3 per body: FP64 (one-sided GI_EPI_SUM launches)
                             // or int64 fixed point (paired far field)
    // The contact pass runs on `aux`, beside the far field on the caller's
    // stream: forked after the previous step, joined before the epilogue.
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // Paired far field, side-by-side path: the far field on `far` (middle
    // priority), the grid build and tiled contacts on `aux` (highest), the
    // warp contact kernel on `aux_lo` (lowest), so that its blocks run in
    // the room the far field's CTAs leave rather than in their place.
    cudaStream_t far = nullptr, aux_lo = nullptr;
    cudaEvent_t ev_far = nullptr, ev_lo = nullptr, ev_grid = nullptr;
};

struct gi_ctx {
    int device = 0;
    int sm_count = 0;
    gi_options opt{GI_SEP_REF_INT, GI_ACCUM_PAIRED, 0, 0};
    bool forced = false;
    gi_tuning forced_tuning{0, 0};
    // Tuned i-bodies per thread per N bucket (floor(log2 n)); 0 = default.
    int bucket_ipt[32] = {0};
    int bucket_shift[32] = {0};  // big-chunk size scale 2^shift of the default
    int bucket_pshift[32] = {0};  // GI_ACCUM_PAIRED: chunks per item scale 2^shift
    std::map<cudaStream_t, StreamScratch> scratch;
    // gi_run_host's device copies of the caller's host state, two pairs
    // that the steps alternate between.
    float4 *mirror_pos = nullptr, *mirror_vel = nullptr;
    float4 *mirror2_pos = nullptr, *mirror2_vel = nullptr;
    size_t mirror_cap = 0;
    // 16 doubles per block of the larger diagnostics grid, 16 for the
    // result, then the passes' two tickets
    double *diag_work = nullptr;
    double *diag_host = nullptr;  // pinned: the result's read-back
    int diag_blocks1 = 0, diag_blocks2 = 0;
    double *pot_buf = nullptr;
    size_t pot_cap = 0;
    int occ[4][9];  // resident one-sided force CTAs per SM: [accum][i-bodies per thread]
};

static int ctx_init(gi_ctx *c, int device)
{
    int ndev = 0;
    GI_CUDA(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) return fail(GI_ERR_NO_DEVICE, "device %d of %d", device, ndev);
    c->device = device;
    cudaDeviceProp prop;
    GI_CUDA(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    if (prop.major != 10 || prop.minor != 3)
        return fail(GI_ERR_NO_DEVICE, "libgi is built for sm_103 only; device %d is sm_%d%d",
                    device, prop.major, prop.minor);
    c->sm_count = prop.multiProcessorCount;
    DeviceGuard g(device);
    c->diag_blocks1 = gi_diag_blocks(1, c->sm_count);  // shared by the two material classes
    c->diag_blocks2 = gi_diag_blocks(2, c->sm_count);
    for (int acc : {GI_ACC_KAHAN, GI_ACC_FP32, GI_ACC_FP64})
        for (int p : {1, 2, 4, 8}) {
            const int o = std::min({gi_force_occupancy(p, acc, GI_EPI_FORCE),
                                    gi_force_occupancy(p, acc, GI_EPI_STEP),
                                    gi_force_occupancy(p, acc, GI_EPI_SUM)});
            c->occ[acc][p] = std::max(o, 1);
        }
    return GI_OK;
}

static void ctx_free(gi_ctx *c)
{
    DeviceGuard g(c->device);
    for (auto &kv : c->scratch) {
        StreamScratch &x = kv.second;
        cudaFree(x.counters);
        cudaFree(x.partials);
        cudaFree(x.pp_pos);
        cudaFree(x.pp_vel);
        cudaFree(x.grid_work);
        cudaFree(x.delta);
        cudaFree(x.fsum);
        if (x.ev_fork) cudaEventDestroy(x.ev_fork);
        if (x.ev_join) cudaEventDestroy(x.ev_join);
        if (x.ev_far) cudaEventDestroy(x.ev_far);
        if (x.ev_lo) cudaEventDestroy(x.ev_lo);
        if (x.ev_grid) cudaEventDestroy(x.ev_grid);
        if (x.aux) cudaStreamDestroy(x.aux);
        if (x.far) cudaStreamDestroy(x.far);
        if (x.aux_lo) cudaStreamDestroy(x.aux_lo);
    }
    c->scratch.clear();
    cudaFree(c->mirror_pos);
    cudaFree(c->mirror_vel);
    cudaFree(c->mirror2_pos);
    cudaFree(c->mirror2_vel);
    cudaFree(c->diag_work);
    cudaFreeHost(c->diag_host);
    cudaFree(c->pot_buf);
}

extern "C" int gi_ctx_create(gi_ctx **out, int device)
{
    if (!out) return fail(GI_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    gi_ctx *c = new gi_ctx();
    int st = ctx_init(c, device);
    if (st != GI_OK) { delete c; return st; }
    *out = c;
    return GI_OK;
}

extern "C" int gi_ctx_destroy(gi_ctx *c)
{
    if (!c) return GI_OK;
    {
        DeviceGuard g(c->device);
        cudaDeviceSynchronize();
    }
    ctx_free(c);
    delete c;
    return GI_OK;
}

extern "C" int gi_ctx_set_options(gi_ctx *c, const gi_options *o)
{
    if (!c || !o) return fail(GI_ERR_INVALID_ARG, "NULL argument");
    if (o->sep_test != GI_SEP_REF_INT && o->sep_test != GI_SEP_SIGN)
        return fail(GI_ERR_INVALID_ARG, "sep_test %d", o->sep_test);
    if (o->accum < GI_ACCUM_PAIRED || o->accum > GI_ACCUM_KAHAN)
        return fail(GI_ERR_INVALID_ARG, "accum %d", o->accum);
    if (o->dense_min < 0) return fail(GI_ERR_INVALID_ARG, "dense_min %d", o->dense_min);
    if (o->cluster_tries < 0) return fail(GI_ERR_INVALID_ARG, "cluster_tries %d", o->cluster_tries);
    c->opt = *o;
    return GI_OK;
}

extern "C" int gi_ctx_set_tuning(gi_ctx *c, const gi_tuning *t)
{
    if (!c) return fail(GI_ERR_INVALID_ARG, "ctx is NULL");
    if (!t) { c->forced = false; return GI_OK; }
    if (t->i_per_thread != 1 && t->i_per_thread != 2 && t->i_per_thread != 4 &&
        t->i_per_thread != 8)
        return fail(GI_ERR_INVALID_ARG, "i_per_thread must be 1, 2, 4 or 8");
    if (t->jchunk < 0 || t->jchunk % 32 != 0 ||
        (t->jchunk > 0 && (t->jchunk / 32 & (t->jchunk / 32 - 1)) != 0))
        return fail(GI_ERR_INVALID_ARG, "jchunk must be 0 or 32 times a power of two");
    c->forced = true;
    c->forced_tuning = *t;
    return GI_OK;
}

static int bucket_of(int n)
{
    int b = 0;
    while ((1 << (b + 1)) <= n && b < 30) ++b;
    return b;
}

// Decomposition of one run: a function of n and the context's tuning table
// only, never of the rest of the batch (results are batch-invariant).
static void tuning_for(const gi_ctx *c, int n, int *ipt, int *jchunk)
{
    if (c->forced) {
        *ipt = c->forced_tuning.i_per_thread;
        int jc = c->forced_tuning.jchunk;
        if (jc <= 0) jc = ((std::max(n, 1) + GI_NT - 1) / GI_NT) * GI_NT;
        *jchunk = std::max(jc, GI_NT);  // the one-sided kernel's chunks are whole tiles
        return;
    }
    const int b = bucket_of(std::max(n, 1));
    int p = c->bucket_ipt[b];
    if (p == 0) p = n >= 262144 ? 2 : 1;
    // Big-chunk size (a power of two of tiles): a big item must be no longer
    // than a quarter of one resident CTA's share of the run, so that the
    // CTAs still have small items to even out their finishing times:
    //   C (tiles) <= 1/4 * T * nib / slots, scaled by the tuned 2^shift.
    // Depends on n and the context's tuning table only, so a run
    // decomposes the same way alone and in any batch.
    const int slots = c->sm_count * c->occ[c->opt.accum][p];
    const int T = (n + GI_NT - 1) / GI_NT;
    const int nib = (n + GI_NT * p - 1) / (GI_NT * p);
    long long ct = std::max(1LL, (long long)T * nib / (4LL * slots));
    const int shift = c->bucket_shift[b];
    ct = shift >= 0 ? (ct << shift) : std::max(1LL, ct >> (-shift));
    int lg = 0;
    while ((2LL << lg) <= ct && (2LL << lg) <= T) ++lg;
    *ipt = p;
    *jchunk = GI_NT << lg;
}

// Chunking of one run: chunks of 2^lg tiles, the last lg shrinking by
// halves to one tile (see tail_tiles in gi_force_impl.cuh).
static void chunking(int n, int jchunk, int *lg, int *tiles, int *nsplit)
{
    const int T = (n + GI_NT - 1) / GI_NT;
    int l = 0;
    while ((GI_NT << (l + 1)) <= jchunk) ++l;
    if ((1LL << l) >= T) {  // one chunk holds the run
        *lg = l;
        *tiles = T;
        *nsplit = 1;
        return;
    }
    int r = 0;
    long long covered = 0;
    while (covered < T) {
        covered = (r + 1 <= l) ? (1LL << (r + 1)) - 1 : (1LL << l) - 1 + (long long)(r + 1 - l) * (1LL << l);
        ++r;
    }
    *lg = l;
    *tiles = T;
    *nsplit = r;
}

// ---- GI_ACCUM_PAIRED decomposition (gi_force_pair.cu): i-blocks of
// kPairRows bodies; block a covers the j-chunks from its own first body to
// the end of the run in work items of 2^pcl chunks.

// Work items of a run of n bodies with 2^pcl chunks per item.
static long long pair_items(int n, int pcl)
{
    const long long C = (n + gi::kPairChunk - 1) / gi::kPairChunk;
    const long long nb = (n + gi::kPairRows - 1) / gi::kPairRows;
    const long long cpi = 1LL << pcl, q = gi::kPairBlockChunks / cpi;
    const long long k0 = (C + cpi - 1) / cpi;
    return nb * k0 - q * (nb * (nb - 1) / 2);
}

static int log2_floor(long long v)
{
    int l = 0;
    while ((2LL << l) <= v) ++l;
    return l;
}

// log2 of the j-chunks per item for a run of n bodies: a function of n and
// the context's tuning table only, never of the rest of the batch.  The
// default spans 256 j-bodies per item below 32,768 bodies (4 chunks of 64),
// 512 below 131,072 and 1,024 above.  Each item ends with 3 global atomics
// per i-body, so items much shorter than that lose to the flush: measured
// with the kernel's earlier 32-body chunks per gi_forces call on uniform
// balls (ms, lone run / 8 runs in one call; j-bodies per item), n = 16,384:
// 256 j 0.126 / 0.713, 512 j 0.113 / 0.736; 25,000: 256 j 0.218 / 1.497;
// 45,000: 512 j 0.624 / 4.407, 1,024 j 0.598 / 4.418; 66,000: 512 j 1.195 /
// 9.218, 256 j 1.199 / 9.338; 100,000: 512 j 2.618 / 20.61; 142,000: 1,024 j
// 5.195 / 40.82; 32 j per item 1.1-1.3x slower at every size.
static int pair_pcl_for(const gi_ctx *c, int n)
{
    const int lmax = log2_floor(gi::kPairMaxCpi);
    if (c->forced) {
        int jc = c->forced_tuning.jchunk;
        if (jc <= 0 || jc > gi::kPairMaxCpi * gi::kPairChunk) jc = gi::kPairMaxCpi * gi::kPairChunk;
        return log2_floor(jc / gi::kPairChunk);
    }
    const int l = gi_internal_pair_default_pcl(n) + c->bucket_pshift[bucket_of(std::max(n, 1))];
    return std::min(std::max(l, 0), lmax);
}

int gi_internal_pair_default_pcl(int n) { return 2 + (n >= 32768) + (n >= 131072); }

extern "C" int gi_ctx_get_tuning(gi_ctx *c, int n, gi_tuning *out)
{
    if (!c || !out) return fail(GI_ERR_INVALID_ARG, "NULL argument");
    if (n < 0) return fail(GI_ERR_BAD_SIZE, "n = %d", n);
    if (c->opt.accum == GI_ACC_PAIRED) {
        out->i_per_thread = gi::kPairIpl;
        out->jchunk = gi::kPairChunk << pair_pcl_for(c, n);
        return GI_OK;
    }
    tuning_for(c, n, &out->i_per_thread, &out->jchunk);
    return GI_OK;
}

// ---------------------------------------------------------------- planning --

struct Plan {
    bool paired = false;  // GI_ACCUM_PAIRED tables (gi_force_pair.cu)
    std::vector<LaunchTable> tables;
    std::vector<int> ipt;
    std::vector<long long> bodies;  // bodies in each table's runs
    std::vector<size_t> ticks;      // split tickets of each table
    size_t tickets = 0;   // max over tables (tables run one after another)
    size_t partials = 0;  // doubles, max over tables
    int max_end = 0;      // largest offset + n
};

static int check_body_ptr(const void *p, const char *name)
{
    if (!p) return fail(GI_ERR_INVALID_ARG, "%s is NULL", name);
    if (reinterpret_cast<uintptr_t>(p) % 16 != 0)
        return fail(GI_ERR_ALIGNMENT, "%s is not 16-byte aligned", name);
    return GI_OK;
}

static int check_runs(const gi_run *runs, int nruns, int nparams)
{
    if (nruns < 0) return fail(GI_ERR_INVALID_ARG, "nruns = %d", nruns);
    if (nruns > 0 && !runs) return fail(GI_ERR_INVALID_ARG, "runs is NULL");
    std::vector<std::pair<long long, long long>> iv;
    for (int r = 0; r < nruns; ++r) {
        const gi_run &q = runs[r];
        if (q.offset < 0 || q.n < 0 || (long long)q.offset + q.n > 0x7fffffffLL)
            return fail(GI_ERR_BAD_SIZE, "run %d: offset %d n %d", r, q.offset, q.n);
        if (q.nfe < 0 || q.nfe > q.n)
            return fail(GI_ERR_BAD_SIZE, "run %d: nfe %d not in [0, %d]", r, q.nfe, q.n);
        if (q.params < 0 || q.params >= nparams)
            return fail(GI_ERR_INVALID_ARG, "run %d: params index %d of %d", r, q.params, nparams);
        if (q.n > 0) iv.push_back({q.offset, (long long)q.offset + q.n});
    }
    std::sort(iv.begin(), iv.end());
    for (size_t k = 1; k < iv.size(); ++k)
        if (iv[k].first < iv[k - 1].second) return fail(GI_ERR_INVALID_ARG, "runs overlap");
    return GI_OK;
}

// Fixed-point unit of a run's paired far-field sums: a power of two such
// that n gm_max^2, a bound on any sum of a body's pair terms
// (|G m_i m_j dp| / max(r, 1)^3 <= gm_max^2), stays below 2^62 units.
static void pair_far_unit(int n, const PairDev &p, RunDev &d)
{
    const double g = std::max(std::fabs((double)p.gm_fe), std::fabs((double)p.gm_si));
    const int e = log2_floor(std::max(n, 2) - 1) + 1;  // 2^e >= n
    int E = (g > 0.0 ? std::ilogb(g * g) + 1 : 0) + e - 62;
    E = std::min(std::max(E, -126), 126);  // 2^-E is a normal float
    d.far_unit = std::ldexp(1.0, E);
    d.far_inv = (float)std::ldexp(1.0, -E);
}

// Stride of a run's item permutation: coprime with the item count, about
// the items of one i-block, so that consecutive CTAs hold different i-blocks.
static int pair_stride(long long items, int nblocks)
{
    if (items <= 1) return 1;
    long long p = std::max(1LL, items / std::max(nblocks, 1));
    auto gcd = [](long long a, long long b) {
        while (b) { const long long r = a % b; a = b; b = r; }
        return a;
    };
    while (gcd(p, items) != 1) ++p;
    return (int)p;
}

long long gi_internal_pair_run(RunDev &d, int n, int pcl, const PairDev &p, long long item_start)
{
    d.ipt = gi::kPairIpl;
    d.pcl = pcl;
    d.pnc = (n + gi::kPairChunk - 1) / gi::kPairChunk;
    d.pnb = (n + gi::kPairRows - 1) / gi::kPairRows;
    d.pk0 = (d.pnc + (1 << pcl) - 1) >> pcl;
    pair_far_unit(n, p, d);
    d.item_start = (int)std::min(item_start, 0x7fffffffLL);
    const long long ri = pair_items(n, pcl);
    d.pitems = (int)std::min(ri, 0x7fffffffLL);
    d.pstride = pair_stride(ri, d.pnb);
    return ri;
}

extern "C" int gi_debug_pair_plan(gi_ctx *c, int n, int pcl_in, long long out[6])
{
    if (!out) return fail(GI_ERR_INVALID_ARG, "out is NULL");
    if (n <= 0) return fail(GI_ERR_BAD_SIZE, "n = %d", n);
    if (pcl_in > log2_floor(gi::kPairMaxCpi)) return fail(GI_ERR_INVALID_ARG, "pcl = %d", pcl_in);
    RunDev d;
    std::memset(&d, 0, sizeof d);
    PairDev p;
    std::memset(&p, 0, sizeof p);
    p.gm_fe = p.gm_si = 1.0f;
    const int pcl = pcl_in >= 0 ? pcl_in : (c ? pair_pcl_for(c, n) : gi_internal_pair_default_pcl(n));
    const long long items = gi_internal_pair_run(d, n, pcl, p, 0);
    out[0] = d.pcl;
    out[1] = d.pnc;
    out[2] = d.pnb;
    out[3] = items;
    out[4] = d.pstride;
    out[5] = d.pk0;
    return GI_OK;
}

static int make_pair_plan(const gi_ctx *c, const gi_run *runs, int nruns,
                          const std::vector<PairDev> &pd, Plan &plan)
{
    plan.paired = true;
    std::vector<int> order;
    for (int r = 0; r < nruns; ++r) {
        if (runs[r].n <= 0) continue;
        order.push_back(r);
        plan.max_end = std::max(plan.max_end, runs[r].offset + runs[r].n);
    }
    // big runs first, so that their CTAs start first
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return runs[a].n > runs[b].n; });
    size_t k = 0;
    while (k < order.size()) {
        LaunchTable t;
        std::memset(&t, 0, sizeof t);
        t.sep_test = c->opt.sep_test;
        t.dense_min = c->opt.dense_min > 0 ? c->opt.dense_min : 256;
        long long items = 0, nb = 0;
        while (k < order.size() && t.nruns < GI_MAX_RUNS) {
            const gi_run &q = runs[order[k]];
            RunDev &d = t.runs[t.nruns++];
            d.offset = q.offset;
            d.n = q.n;
            d.nfe = q.nfe;
            d.param = q.params;
            items += gi_internal_pair_run(d, q.n, pair_pcl_for(c, q.n), pd[q.params], items);
            nb += q.n;
            d.dt = q.dt;
            d.dtm_fe = q.dt_over_mass_fe;
            d.dtm_si = q.dt_over_mass_si;
            d.damp = q.damp;
            ++k;
        }
        if (items > 0x7fffffffLL) return fail(GI_ERR_BAD_SIZE, "too many work items");
        t.nitems = (int)items;
        for (size_t m = 0; m < pd.size(); ++m) t.params[m] = pd[m];
        plan.tables.push_back(t);
        plan.ipt.push_back(gi::kPairIpl);
        plan.bodies.push_back(nb);
        plan.ticks.push_back(0);
    }
    return GI_OK;
}

static int make_plan(const gi_ctx *c, const gi_run *runs, int nruns,
                     const std::vector<PairDev> &pd, Plan &plan)
{
    if (c->opt.accum == GI_ACC_PAIRED) return make_pair_plan(c, runs, nruns, pd, plan);
    // Group runs by i-bodies-per-thread (one kernel instance per group), big
    // runs first so their CTAs start first.
    std::vector<int> order;
    std::vector<int> ipt(nruns), jc(nruns);
    for (int r = 0; r < nruns; ++r) {
        if (runs[r].n <= 0) continue;
        tuning_for(c, runs[r].n, &ipt[r], &jc[r]);
        order.push_back(r);
        plan.max_end = std::max(plan.max_end, runs[r].offset + runs[r].n);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (ipt[a] != ipt[b]) return ipt[a] > ipt[b];
        return runs[a].n > runs[b].n;
    });
    size_t k = 0;
    while (k < order.size()) {
        LaunchTable t;
        std::memset(&t, 0, sizeof t);
        t.sep_test = c->opt.sep_test;
        t.dense_min = c->opt.dense_min > 0 ? c->opt.dense_min : 256;
        const int p = ipt[order[k]];
        long long items = 0, tick = 0, part = 0, nb = 0;
        while (k < order.size() && ipt[order[k]] == p && t.nruns < GI_MAX_RUNS) {
            const gi_run &q = runs[order[k]];
            RunDev &d = t.runs[t.nruns++];
            d.offset = q.offset;
            d.n = q.n;
            d.nfe = q.nfe;
            d.param = q.params;
            d.jchunk = jc[order[k]];
            chunking(q.n, d.jchunk, &d.lg, &d.tiles, &d.nsplit);
            d.nib = (q.n + GI_NT * p - 1) / (GI_NT * p);
            d.ipt = p;
            d.item_start = (int)items;
            items += (long long)d.nib * d.nsplit;
            nb += q.n;
            if (d.nsplit > 1) {
                d.tick_base = (int)tick;
                d.part_base = part;
                tick += d.nib;
                part += (long long)d.nsplit * 3 * q.n;
            }
            d.dt = q.dt;
            d.dtm_fe = q.dt_over_mass_fe;
            d.dtm_si = q.dt_over_mass_si;
            d.damp = q.damp;
            ++k;
        }
        if (items > 0x7fffffffLL) return fail(GI_ERR_BAD_SIZE, "too many work items");
        t.nitems = (int)items;
        for (size_t m = 0; m < pd.size(); ++m) t.params[m] = pd[m];
        plan.tables.push_back(t);
        plan.ipt.push_back(p);
        plan.bodies.push_back(nb);
        plan.ticks.push_back((size_t)tick);
        plan.tickets = std::max(plan.tickets, (size_t)tick);
        plan.partials = std::max(plan.partials, (size_t)part);
    }
    return GI_OK;
}

static bool stream_capturing(cudaStream_t s)
{
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) != cudaSuccess) return false;
    return st != cudaStreamCaptureStatusNone;
}

static int ensure_scratch(gi_ctx *c, const Plan &plan, cudaStream_t s, StreamScratch **out)
{
    StreamScratch &x = c->scratch[s];
    *out = &x;
    const bool grow_t = plan.tickets > x.tickets_cap;
    const bool grow_p = plan.partials > x.partials_cap;
    size_t gwords = 0;
    for (long long b : plan.bodies) gwords = std::max(gwords, gi_grid_words(plan.max_end, b));
    const bool grow_g = gwords > x.grid_work_cap;
    const bool grow_d = (size_t)plan.max_end > x.delta_cap;
    if (!grow_t && !grow_p && !grow_g && !grow_d && x.counters && x.aux) return GI_OK;
    if (stream_capturing(s))
        return fail(GI_ERR_INVALID_ARG,
                    "scratch must grow (run once outside stream capture before capturing)");
    GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (!x.aux) {
        int lo = 0, hi = 0;  // hi: the greatest priority (numerically lowest)
        GI_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi), "cudaDeviceGetStreamPriorityRange");
        GI_CUDA(cudaStreamCreateWithPriority(&x.aux, cudaStreamNonBlocking, hi),
                "cudaStreamCreateWithPriority");
        GI_CUDA(cudaEventCreateWithFlags(&x.ev_fork, cudaEventDisableTiming), "cudaEventCreate");
        GI_CUDA(cudaEventCreateWithFlags(&x.ev_join, cudaEventDisableTiming), "cudaEventCreate");
        GI_CUDA(cudaStreamCreateWithPriority(&x.far, cudaStreamNonBlocking, (lo + hi) / 2),
                "cudaStreamCreateWithPriority");
        GI_CUDA(cudaStreamCreateWithPriority(&x.aux_lo, cudaStreamNonBlocking, lo),
                "cudaStreamCreateWithPriority");
        GI_CUDA(cudaEventCreateWithFlags(&x.ev_far, cudaEventDisableTiming), "cudaEventCreate");
        GI_CUDA(cudaEventCreateWithFlags(&x.ev_lo, cudaEventDisableTiming), "cudaEventCreate");
        GI_CUDA(cudaEventCreateWithFlags(&x.ev_grid, cudaEventDisableTiming), "cudaEventCreate");
    }
    if (grow_t || !x.counters) {
        cudaFree(x.counters);
        x.counters = x.queue = x.tickets = nullptr;
        x.tickets_cap = 0;
        size_t cap = std::max(plan.tickets, (size_t)1024);
        GI_CUDA(cudaMalloc(&x.counters, (cap + 2) * sizeof(unsigned int)), "cudaMalloc counters");
        GI_CUDA(cudaMemset(x.counters, 0, (cap + 2) * sizeof(unsigned int)), "cudaMemset counters");
        x.queue = x.counters;
        x.tickets = x.counters + 2;
        x.tickets_cap = cap;
    }
    if (grow_p) {
        cudaFree(x.partials);
        x.partials = nullptr;
        x.partials_cap = 0;
        size_t cap = plan.partials + plan.partials / 4;
        GI_CUDA(cudaMalloc(&x.partials, cap * sizeof(double)), "cudaMalloc partials");
        x.partials_cap = cap;
    }
    if (grow_g) {
        cudaFree(x.grid_work);
        x.grid_work = nullptr;
        x.grid_work_cap = 0;
        GI_CUDA(cudaMalloc(&x.grid_work, gwords * sizeof(unsigned int)), "cudaMalloc grid");
        x.grid_work_cap = gwords;
    }
    if (grow_d) {
        cudaFree(x.delta);
        cudaFree(x.fsum);
        x.delta = nullptr;
        x.fsum = nullptr;
        x.delta_cap = 0;
        GI_CUDA(cudaMalloc(&x.delta, (size_t)plan.max_end * 3 * sizeof(long long)), "cudaMalloc delta");
        GI_CUDA(cudaMalloc(&x.fsum, (size_t)plan.max_end * 3 * sizeof(double)), "cudaMalloc fsum");
        x.delta_cap = plan.max_end;
    }
    return GI_OK;
}

static int convert_params(const gi_pair_params *params, int nparams, std::vector<PairDev> &pd)
{
    if (nparams < 1 || nparams > GI_MAX_PARAMS)
        return fail(GI_ERR_BAD_SIZE, "nparams = %d (1..%d)", nparams, GI_MAX_PARAMS);
    if (!params) return fail(GI_ERR_INVALID_ARG, "params is NULL");
    pd.resize(nparams);
    for (int m = 0; m < nparams; ++m) {
        int st = to_device_params(params[m], pd[m]);
        if (st != GI_OK) return st;
    }
    return GI_OK;
}

// Tables of fewer than kOverlapMaxPairs pairs (sum of n^2 over their runs)
// run the contact pass beside the far field.  Larger ones, where the contact
// pass is a sliver of the step and the far field wants every resident CTA,
// run it first and take the fused epilogue.  Measured with gi_forces on
// uniform balls (default tuning): the side-by-side pass takes 33 % off at
// n = 8,192, 5 % at 49,152, 2 % at 98,304, and adds 5 % at 131,072.
constexpr long long kOverlapMaxPairs = 1LL << 34;
// Far-field CTAs per SM while the contact pass runs beside it.  Measured on
// the 66,000-body impact (ms per fused step, settled / collision phase):
// 3 CTAs 1.72 / 2.60, 4: 1.68 / 2.57, 6: 1.68 / 2.59, 8: 1.67 / 2.54; the
// contact kernels fit beside 8 of them, and more warps keep the far field's
// FMA pipe busier.
constexpr int kSideBySideCtas = 8;

// One force evaluation (or fused step) per table.  The contact pass and the
// far field are independent until the epilogue, so for tables of fewer than
// kOverlapMaxPairs pairs they run side by side, forked from the caller's
// stream with events and joined before the epilogue:
//   - paired far field (the default): the far field on the scratch's
//     middle-priority stream, the grid build and the tiled contacts on the
//     highest-priority one, the warp contacts on the lowest (their small
//     blocks fill the registers the far field's CTAs leave free);
//   - one-sided modes: the contact pass on the aux stream, the far field on
//     the caller's stream with kSideBySideCtas resident CTAs per SM (at that
//     size it runs as fast as at full occupancy and leaves room on every SM
//     for the contact kernels).
// The epilogue then runs on the caller's stream with the fused epilogue's
// arithmetic.  Larger tables run the contact pass first.  Either way the
// results are the same bits.
static int run_force_plan(gi_ctx *c, const StreamScratch *x, const Plan &plan, int epi,
                          const float4 *pos, const float4 *vel, float4 *force,
                          float4 *pos_out, float4 *vel_out, cudaStream_t s)
{
    for (size_t t = 0; t < plan.tables.size(); ++t) {
        const LaunchTable &tab = plan.tables[t];
        ForceArgs a;
        a.pos = pos;
        a.vel = vel;
        a.force = force;
        a.pos_out = pos_out;
        a.vel_out = vel_out;
        a.partials = x->partials;
        a.tickets = x->tickets;
        a.queue = x->queue;
        a.delta = x->delta;
        a.fsum = x->fsum;
        a.fsum_fx = nullptr;
        int maxn = 0;
        long long pairs = 0;
        for (int r = 0; r < tab.nruns; ++r) {
            maxn = std::max(maxn, tab.runs[r].n);
            pairs += (long long)tab.runs[r].n * tab.runs[r].n;
        }
        if (plan.paired) {
            // The far-field sums start at zero; captured with the launches
            // when the stream is capturing.
            a.fsum_fx = reinterpret_cast<long long *>(x->fsum);
            GI_CUDA(cudaMemsetAsync(a.fsum_fx, 0, (size_t)plan.max_end * 3 * sizeof(long long), s),
                    "cudaMemsetAsync far-field sums");
            if (pairs >= kOverlapMaxPairs) {
                GI_CUDA(gi_launch_contacts(pos, vel, tab, plan.bodies[t], plan.max_end,
                                           x->grid_work, x->delta, c->sm_count, s),
                        "contact pass");
                GI_CUDA(gi_launch_pair_force(a, tab, s), "paired force kernel launch");
            } else {
                // The far field is launched first: it is the long kernel, and
                // a synchronous caller would otherwise wait for the contact
                // pass's dozen launches before it starts.
                GI_CUDA(cudaEventRecord(x->ev_fork, s), "cudaEventRecord");
                GI_CUDA(cudaStreamWaitEvent(x->far, x->ev_fork, 0), "cudaStreamWaitEvent");
                GI_CUDA(cudaStreamWaitEvent(x->aux, x->ev_fork, 0), "cudaStreamWaitEvent");
                GI_CUDA(gi_launch_pair_force(a, tab, x->far), "paired force kernel launch");
                GI_CUDA(cudaEventRecord(x->ev_far, x->far), "cudaEventRecord");
                GI_CUDA(gi_launch_contacts(pos, vel, tab, plan.bodies[t], plan.max_end,
                                           x->grid_work, x->delta, c->sm_count, x->aux,
                                           x->aux_lo, x->ev_grid),
                        "contact pass");
                GI_CUDA(cudaEventRecord(x->ev_join, x->aux), "cudaEventRecord");
                GI_CUDA(cudaEventRecord(x->ev_lo, x->aux_lo), "cudaEventRecord");
                GI_CUDA(cudaStreamWaitEvent(s, x->ev_far, 0), "cudaStreamWaitEvent");
                GI_CUDA(cudaStreamWaitEvent(s, x->ev_join, 0), "cudaStreamWaitEvent");
                GI_CUDA(cudaStreamWaitEvent(s, x->ev_lo, 0), "cudaStreamWaitEvent");
            }
            GI_CUDA(gi_launch_pair_finish(epi, a, tab, maxn, c->sm_count, s), "epilogue launch");
            continue;
        }
        const int p = plan.ipt[t];
        const int occ = c->occ[c->opt.accum][p];
        // The queue and this table's tickets start at zero (the kernel also
        // re-arms them on the way out; this covers a launch that never got
        // there).  Captured with the launch when the stream is capturing.
        GI_CUDA(cudaMemsetAsync(x->counters, 0, (2 + plan.ticks[t]) * sizeof(unsigned int), s),
                "cudaMemsetAsync counters");
        if (pairs >= kOverlapMaxPairs) {
            GI_CUDA(gi_launch_contacts(pos, vel, tab, plan.bodies[t], plan.max_end, x->grid_work,
                                       x->delta, c->sm_count, s),
                    "contact pass");
            GI_CUDA(gi_launch_force(p, c->opt.accum, epi, a, tab, c->sm_count * occ, s),
                    "force kernel launch");
            continue;
        }
        GI_CUDA(cudaEventRecord(x->ev_fork, s), "cudaEventRecord");
        GI_CUDA(cudaStreamWaitEvent(x->aux, x->ev_fork, 0), "cudaStreamWaitEvent");
        GI_CUDA(gi_launch_contacts(pos, vel, tab, plan.bodies[t], plan.max_end, x->grid_work,
                                   x->delta, c->sm_count, x->aux),
                "contact pass");
        GI_CUDA(cudaEventRecord(x->ev_join, x->aux), "cudaEventRecord");
        GI_CUDA(gi_launch_force(p, c->opt.accum, GI_EPI_SUM, a, tab,
                                c->sm_count * std::min(occ, kSideBySideCtas), s),
                "force kernel launch");
        GI_CUDA(cudaStreamWaitEvent(s, x->ev_join, 0), "cudaStreamWaitEvent");
        GI_CUDA(gi_launch_finish(epi, a, tab, maxn, c->sm_count, s), "epilogue launch");
    }
    return GI_OK;
}

// ------------------------------------------------------------- entry points --

extern "C" int gi_forces(gi_ctx *c, const float *pos, const float *vel, float *force,
                         const gi_run *runs, int nruns, const gi_pair_params *params,
                         int nparams, void *stream)
{
    if (!c) return fail(GI_ERR_INVALID_ARG, "ctx is NULL");
    int st = check_runs(runs, nruns, nparams);
    if (st) return st;
    std::vector<PairDev> pd;
    if ((st = convert_params(params, nparams, pd))) return st;
    Plan plan;
    if ((st = make_plan(c, runs, nruns, pd, plan))) return st;
    if (plan.tables.empty()) return GI_OK;
    if ((st = check_body_ptr(pos, "pos")) || (st = check_body_ptr(vel, "vel")) ||
        (st = check_body_ptr(force, "force")))
        return st;
    DeviceGuard g(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    StreamScratch *x = nullptr;
    if ((st = ensure_scratch(c, plan, s, &x))) return st;
    return run_force_plan(c, x, plan, GI_EPI_FORCE, (const float4 *)pos, (const float4 *)vel,
                          (float4 *)force, nullptr, nullptr, s);
}

static int move_tables(const gi_run *runs, int nruns, std::vector<LaunchTable> &out)
{
    int k = 0;
    while (k < nruns) {
        LaunchTable t;
        std::memset(&t, 0, sizeof t);
        while (k < nruns && t.nruns < GI_MAX_RUNS) {
            const gi_run &q = runs[k++];
            if (q.n <= 0) continue;
            RunDev &d = t.runs[t.nruns++];
            d.offset = q.offset;
            d.n = q.n;
            d.nfe = q.nfe;
            d.param = q.params;
            d.dt = q.dt;
            d.dtm_fe = q.dt_over_mass_fe;
            d.dtm_si = q.dt_over_mass_si;
            d.damp = q.damp;
        }
        if (t.nruns) out.push_back(t);
    }
    return GI_OK;
}

static int move_impl(float *pos, float *vel, const float *force, const gi_run *runs,
                     int nruns, cudaStream_t s)
{
    std::vector<LaunchTable> tabs;
    move_tables(runs, nruns, tabs);
    if (tabs.empty()) return GI_OK;
    int st;
    if ((st = check_body_ptr(pos, "pos")) || (st = check_body_ptr(vel, "vel")) ||
        (st = check_body_ptr(force, "force")))
        return st;
    for (auto &t : tabs)
        GI_CUDA(gi_launch_move((float4 *)pos, (float4 *)vel, (const float4 *)force, t, s),
                "move kernel launch");
    return GI_OK;
}

extern "C" int gi_move(gi_ctx *c, float *pos, float *vel, const float *force,
                       const gi_run *runs, int nruns, void *stream)
{
    if (!c) return fail(GI_ERR_INVALID_ARG, "ctx is NULL");
    int st = check_runs(runs, nruns, 0x7fffffff);
    if (st) return st;
    DeviceGuard g(c->device);
    return move_impl(pos, vel, force, runs, nruns, (cudaStream_t)stream);
}

static int ensure_pingpong(StreamScratch *x, size_t bodies, cudaStream_t s)
{
    if (bodies <= x->pp_cap) return GI_OK;
    if (stream_capturing(s))
        return fail(GI_ERR_INVALID_ARG,
                    "state buffers must grow (run once outside stream capture before capturing)");
    GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    cudaFree(x->pp_pos);
    cudaFree(x->pp_vel);
    x->pp_pos = x->pp_vel = nullptr;
    x->pp_cap = 0;
    GI_CUDA(cudaMalloc(&x->pp_pos, bodies * sizeof(float4)), "cudaMalloc state");
    GI_CUDA(cudaMalloc(&x->pp_vel, bodies * sizeof(float4)), "cudaMalloc state");
    x->pp_cap = bodies;
    return GI_OK;
}

extern "C" int gi_step(gi_ctx *c, float *pos, float *vel, const gi_run *runs, int nruns,
                       const gi_pair_params *params, int nparams, int nsteps, void *stream)
{
    if (!c) return fail(GI_ERR_INVALID_ARG, "ctx is NULL");
    if (nsteps < 0) return fail(GI_ERR_INVALID_ARG, "nsteps = %d", nsteps);
    int st = check_runs(runs, nruns, nparams);
    if (st) return st;
    std::vector<PairDev> pd;
    if ((st = convert_params(params, nparams, pd))) return st;
    Plan plan;
    if ((st = make_plan(c, runs, nruns, pd, plan))) return st;
    if (plan.tables.empty() || nsteps == 0) return GI_OK;
    if ((st = check_body_ptr(pos, "pos")) || (st = check_body_ptr(vel, "vel"))) return st;
    DeviceGuard g(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    StreamScratch *x = nullptr;
    if ((st = ensure_scratch(c, plan, s, &x))) return st;
    if ((st = ensure_pingpong(x, (size_t)plan.max_end, s))) return st;
    float4 *ip = (float4 *)pos, *iv = (float4 *)vel, *op = x->pp_pos, *ov = x->pp_vel;
    for (int k = 0; k < nsteps; ++k) {
        if ((st = run_force_plan(c, x, plan, GI_EPI_STEP, ip, iv, nullptr, op, ov, s))) return st;
        std::swap(ip, op);
        std::swap(iv, ov);
    }
    if (ip != (float4 *)pos) {
        for (int r = 0; r < nruns; ++r) {
            if (runs[r].n <= 0) continue;
            const size_t off = runs[r].offset, bytes = (size_t)runs[r].n * sizeof(float4);
            GI_CUDA(cudaMemcpyAsync((float4 *)pos + off, ip + off, bytes, cudaMemcpyDeviceToDevice, s),
                    "copy back pos");
            GI_CUDA(cudaMemcpyAsync((float4 *)vel + off, iv + off, bytes, cudaMemcpyDeviceToDevice, s),
                    "copy back vel");
        }
    }
    return GI_OK;
}

extern "C" int gi_step_pingpong(gi_ctx *c, float *pos_a, float *vel_a, float *pos_b,
                                float *vel_b, const gi_run *runs, int nruns,
                                const gi_pair_params *params, int nparams, int nsteps,
                                void *stream)
{
    if (!c) return fail(GI_ERR_INVALID_ARG, "ctx is NULL");
    if (nsteps < 0) return fail(GI_ERR_INVALID_ARG, "nsteps = %d", nsteps);
    int st = check_runs(runs, nruns, nparams);
    if (st) return st;
    std::vector<PairDev> pd;
    if ((st = convert_params(params, nparams, pd))) return st;
    Plan plan;
    if ((st = make_plan(c, runs, nruns, pd, plan))) return st;
    if (plan.tables.empty() || nsteps == 0) return GI_OK;
    if ((st = check_body_ptr(pos_a, "pos_a")) || (st = check_body_ptr(vel_a, "vel_a")) ||
        (st = check_body_ptr(pos_b, "pos_b")) || (st = check_body_ptr(vel_b, "vel_b")))
        return st;
    if (pos_a == pos_b || vel_a == vel_b)
        return fail(GI_ERR_INVALID_ARG, "the two state buffers must differ");
    DeviceGuard g(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    StreamScratch *x = nullptr;
    if ((st = ensure_scratch(c, plan, s, &x))) return st;
    float4 *ip = (float4 *)pos_a, *iv = (float4 *)vel_a, *op = (float4 *)pos_b,
           *ov = (float4 *)vel_b;
    for (int k = 0; k < nsteps; ++k) {
        if ((st = run_force_plan(c, x, plan, GI_EPI_STEP, ip, iv, nullptr, op, ov, s))) return st;
        std::swap(ip, op);
        std::swap(iv, ov);
    }
    return GI_OK;
}

// Autotuner: for each N bucket present in `runs` (its largest run stands for
// it), time the force pass for every decomposition of the context's
// accumulation mode (one-sided: i-bodies per thread and big-chunk scale;
// paired: chunks per item) on the caller's own bodies, and keep the fastest
// in the context's table.  Synchronous; allocates a scratch force array for
// the timing.
extern "C" int gi_autotune(gi_ctx *c, const float *pos, const float *vel, const gi_run *runs,
                           int nruns, const gi_pair_params *params, int nparams, void *stream)
{
    if (!c) return fail(GI_ERR_INVALID_ARG, "ctx is NULL");
    int st = check_runs(runs, nruns, nparams);
    if (st) return st;
    if (stream_capturing((cudaStream_t)stream))
        return fail(GI_ERR_INVALID_ARG, "gi_autotune cannot run under stream capture");
    DeviceGuard g(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    int rep[32];
    for (int b = 0; b < 32; ++b) rep[b] = -1;
    int max_end = 0;
    for (int r = 0; r < nruns; ++r) {
        if (runs[r].n <= 0) continue;
        const int b = bucket_of(runs[r].n);
        if (rep[b] < 0 || runs[r].n > runs[rep[b]].n) rep[b] = r;
        max_end = std::max(max_end, runs[r].offset + runs[r].n);
    }
    if (max_end == 0) return GI_OK;
    const bool was_forced = c->forced;
    c->forced = false;
    float *force = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t ce = cudaMalloc(&force, (size_t)max_end * sizeof(float4));
    if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cudaFree(force);
        c->forced = was_forced;
        return cuda_fail(ce, "autotune setup");
    }
    const bool paired = c->opt.accum == GI_ACC_PAIRED;
    for (int b = 0; b < 32 && st == GI_OK && paired; ++b) {
        // paired far field: the chunks per item, 2^-2 .. 2^2 times the default
        if (rep[b] < 0) continue;
        const gi_run &q = runs[rep[b]];
        float best = 1e30f;
        int best_s = 0;
        for (int sh = -2; sh <= 2 && st == GI_OK; ++sh) {
            c->bucket_pshift[b] = sh;
            st = gi_forces(c, pos, vel, force, &q, 1, params, nparams, stream);
            if (st) break;
            cudaEventRecord(e0, s);
            for (int rep2 = 0; rep2 < 2 && st == GI_OK; ++rep2)
                st = gi_forces(c, pos, vel, force, &q, 1, params, nparams, stream);
            cudaEventRecord(e1, s);
            if (st) break;
            ce = cudaEventSynchronize(e1);
            if (ce != cudaSuccess) { st = cuda_fail(ce, "autotune timing"); break; }
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) { best = ms; best_s = sh; }
        }
        c->bucket_pshift[b] = best_s;
    }
    for (int b = 0; b < 32 && st == GI_OK && !paired; ++b) {
        if (rep[b] < 0) continue;
        const gi_run &q = runs[rep[b]];
        const bool big = q.n > 262144;
        const int ipts[3] = {1, 2, 4};
        float best = 1e30f;
        int best_p = 1, best_s = 0;
        for (int pi = 0; pi < (big ? 2 : 3) && st == GI_OK; ++pi) {
            for (int sh = (big ? -1 : -2); sh <= (big ? 1 : 2) && st == GI_OK; ++sh) {
                c->bucket_ipt[b] = ipts[pi];
                c->bucket_shift[b] = sh;
                // warm-up (also grows scratch), then two timed passes
                st = gi_forces(c, pos, vel, force, &q, 1, params, nparams, stream);
                if (st) break;
                cudaEventRecord(e0, s);
                for (int rep2 = 0; rep2 < 2 && st == GI_OK; ++rep2)
                    st = gi_forces(c, pos, vel, force, &q, 1, params, nparams, stream);
                cudaEventRecord(e1, s);
                if (st) break;
                ce = cudaEventSynchronize(e1);
                if (ce != cudaSuccess) { st = cuda_fail(ce, "autotune timing"); break; }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best) { best = ms; best_p = ipts[pi]; best_s = sh; }
            }
        }
        c->bucket_ipt[b] = best_p;
        c->bucket_shift[b] = best_s;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(force);
    c->forced = was_forced;
    return st;
}

extern "C" int gi_run_host(gi_ctx *c, float *pos_host, float *vel_host, int ntotal,
                           const gi_run *runs, int nruns, const gi_pair_params *params,
                           int nparams, int nsteps, void *stream)
{
    if (!c) return fail(GI_ERR_INVALID_ARG, "ctx is NULL");
    if (!pos_host || !vel_host) return fail(GI_ERR_INVALID_ARG, "host buffer is NULL");
    if (ntotal < 0) return fail(GI_ERR_BAD_SIZE, "ntotal = %d", ntotal);
    int st = check_runs(runs, nruns, nparams);
    if (st) return st;
    for (int r = 0; r < nruns; ++r)
        if (runs[r].offset + runs[r].n > ntotal)
            return fail(GI_ERR_BAD_SIZE, "run %d ends beyond ntotal", r);
    if (ntotal == 0) return GI_OK;
    DeviceGuard g(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    if ((size_t)ntotal > c->mirror_cap) {
        GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        cudaFree(c->mirror_pos);
        cudaFree(c->mirror_vel);
        cudaFree(c->mirror2_pos);
        cudaFree(c->mirror2_vel);
        c->mirror_pos = c->mirror_vel = c->mirror2_pos = c->mirror2_vel = nullptr;
        c->mirror_cap = 0;
        GI_CUDA(cudaMalloc(&c->mirror_pos, ntotal * sizeof(float4)), "cudaMalloc mirror");
        GI_CUDA(cudaMalloc(&c->mirror_vel, ntotal * sizeof(float4)), "cudaMalloc mirror");
        GI_CUDA(cudaMalloc(&c->mirror2_pos, ntotal * sizeof(float4)), "cudaMalloc mirror");
        GI_CUDA(cudaMalloc(&c->mirror2_vel, ntotal * sizeof(float4)), "cudaMalloc mirror");
        c->mirror_cap = ntotal;
    }
    // Only the runs' bodies go to the device and back (contiguous runs as one
    // copy); the rest of the host arrays is neither read nor changed.
    std::vector<std::pair<int, int>> rng;
    for (int r = 0; r < nruns; ++r)
        if (runs[r].n > 0) rng.push_back({runs[r].offset, runs[r].offset + runs[r].n});
    std::sort(rng.begin(), rng.end());
    std::vector<std::pair<int, int>> merged;
    for (const auto &q : rng) {
        if (!merged.empty() && q.first == merged.back().second) merged.back().second = q.second;
        else merged.push_back(q);
    }
    float4 *const hp = reinterpret_cast<float4 *>(pos_host), *const hv = reinterpret_cast<float4 *>(vel_host);
    for (const auto &q : merged) {
        const size_t off = (size_t)q.first, bytes = (size_t)(q.second - q.first) * sizeof(float4);
        GI_CUDA(cudaMemcpyAsync(c->mirror_pos + off, hp + off, bytes, cudaMemcpyHostToDevice, s),
                "H2D pos");
        GI_CUDA(cudaMemcpyAsync(c->mirror_vel + off, hv + off, bytes, cudaMemcpyHostToDevice, s),
                "H2D vel");
    }
    // Steps alternate between the two device pairs, and the result is read
    // back from the pair that holds it (no device-to-device copy).
    if (nsteps > 0 && !merged.empty()) {
        st = gi_step_pingpong(c, (float *)c->mirror_pos, (float *)c->mirror_vel,
                              (float *)c->mirror2_pos, (float *)c->mirror2_vel, runs, nruns,
                              params, nparams, nsteps, stream);
        if (st) return st;
    }
    const float4 *rp = (nsteps & 1) ? c->mirror2_pos : c->mirror_pos;
    const float4 *rv = (nsteps & 1) ? c->mirror2_vel : c->mirror_vel;
    for (const auto &q : merged) {
        const size_t off = (size_t)q.first, bytes = (size_t)(q.second - q.first) * sizeof(float4);
        GI_CUDA(cudaMemcpyAsync(hp + off, rp + off, bytes, cudaMemcpyDeviceToHost, s), "D2H pos");
        GI_CUDA(cudaMemcpyAsync(hv + off, rv + off, bytes, cudaMemcpyDeviceToHost, s), "D2H vel");
    }
    GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    return GI_OK;
}

extern "C" int gi_diag_fp64(gi_ctx *c, const float *pos, const float *vel,
                            const unsigned char *label, int scope, const gi_run *run,
                            const gi_pair_params *params, double *out, void *stream)
{
    if (!c || !run || !params || !out) return fail(GI_ERR_INVALID_ARG, "NULL argument");
    if (scope < 0 || scope > 4) return fail(GI_ERR_INVALID_ARG, "scope %d", scope);
    gi_run q = *run;
    q.params = 0;
    int st = check_runs(&q, 1, 1);
    if (st) return st;
    if ((st = check_body_ptr(pos, "pos")) || (st = check_body_ptr(vel, "vel"))) return st;
    DeviceGuard g(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nbmax = (size_t)std::max(c->diag_blocks1, c->diag_blocks2);
    if (!c->diag_work) {
        GI_CUDA(cudaMalloc(&c->diag_work, (nbmax + 2) * 16 * sizeof(double)), "cudaMalloc diag");
    }
    if (!c->diag_host) {
        GI_CUDA(cudaMallocHost(&c->diag_host, 16 * sizeof(double)), "cudaMallocHost diag");
    }
    double *out_dev = c->diag_work + nbmax * 16;
    int *ticket = (int *)(c->diag_work + (nbmax + 1) * 16);
    RunDev rd;
    std::memset(&rd, 0, sizeof rd);
    rd.offset = q.offset;
    rd.n = q.n;
    rd.nfe = q.nfe;
    GI_CUDA(gi_launch_diag((const float4 *)pos, (const float4 *)vel, label, scope, rd,
                           params->MassFe, params->MassSi, c->diag_work, c->diag_blocks1,
                           c->diag_blocks2, out_dev, ticket, s),
            "diag launch");
    // through pinned memory: a copy into the caller's pageable buffer would
    // be staged by the driver
    GI_CUDA(cudaMemcpyAsync(c->diag_host, out_dev, 15 * sizeof(double), cudaMemcpyDeviceToHost, s),
            "D2H diag");
    GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    std::memcpy(out, c->diag_host, 15 * sizeof(double));
    return GI_OK;
}

extern "C" int gi_potential_fp64(gi_ctx *c, const float *pos, const gi_run *runs, int nruns,
                                 const gi_pair_params *params, int nparams, double *out,
                                 void *stream)
{
    if (!c || !out) return fail(GI_ERR_INVALID_ARG, "NULL argument");
    int st = check_runs(runs, nruns, nparams);
    if (st) return st;
    std::vector<PairDev> pd;
    if ((st = convert_params(params, nparams, pd))) return st;
    for (int r = 0; r < nruns; ++r) out[r] = 0.0;
    if ((st = check_body_ptr(pos, "pos"))) return st;
    DeviceGuard g(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<double> host;
    for (int r0 = 0; r0 < nruns; r0 += GI_MAX_RUNS) {
        LaunchTable t;
        std::memset(&t, 0, sizeof t);
        std::vector<int> idx;
        int blocks = 0;
        for (int r = r0; r < std::min(nruns, r0 + GI_MAX_RUNS); ++r) {
            if (runs[r].n <= 0) continue;
            RunDev &d = t.runs[t.nruns++];
            d.offset = runs[r].offset;
            d.n = runs[r].n;
            d.nfe = runs[r].nfe;
            d.param = runs[r].params;
            d.item_start = blocks;
            blocks += (runs[r].n + GI_NT - 1) / GI_NT;
            idx.push_back(r);
        }
        if (!t.nruns) continue;
        t.nitems = blocks;
        for (size_t m = 0; m < pd.size(); ++m) t.params[m] = pd[m];
        if ((size_t)blocks > c->pot_cap) {
            GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
            cudaFree(c->pot_buf);
            c->pot_buf = nullptr;
            c->pot_cap = 0;
            GI_CUDA(cudaMalloc(&c->pot_buf, (size_t)blocks * sizeof(double)), "cudaMalloc potential");
            c->pot_cap = blocks;
        }
        GI_CUDA(gi_launch_potential((const float4 *)pos, t, c->pot_buf, blocks, s), "potential launch");
        host.resize(blocks);
        GI_CUDA(cudaMemcpyAsync(host.data(), c->pot_buf, (size_t)blocks * sizeof(double),
                                cudaMemcpyDeviceToHost, s),
                "D2H potential");
        GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        for (int k = 0; k < t.nruns; ++k) {
            const int b0 = t.runs[k].item_start;
            const int b1 = (k + 1 < t.nruns) ? t.runs[k + 1].item_start : blocks;
            double u = 0.0;
            for (int b = b0; b < b1; ++b) u += host[b];
            out[idx[k]] = u;
        }
    }
    return GI_OK;
}

extern "C" int gi_debug_fill_counters(gi_ctx *c, void *stream, unsigned int value)
{
    if (!c) return fail(GI_ERR_INVALID_ARG, "ctx is NULL");
    auto it = c->scratch.find((cudaStream_t)stream);
    if (it == c->scratch.end() || !it->second.counters)
        return fail(GI_ERR_INVALID_ARG, "no force scratch on this stream yet");
    DeviceGuard g(c->device);
    StreamScratch &x = it->second;
    const size_t words = x.tickets_cap + 2;
    const unsigned char b = (unsigned char)(value & 0xffu);
    if (value != 0x01010101u * b)
        return fail(GI_ERR_INVALID_ARG, "value must repeat one byte (a memset pattern)");
    GI_CUDA(cudaMemsetAsync(x.counters, b, words * sizeof(unsigned int), (cudaStream_t)stream),
            "cudaMemsetAsync");
    GI_CUDA(cudaStreamSynchronize((cudaStream_t)stream), "cudaStreamSynchronize");
    return GI_OK;
}

extern "C" int gi_measure_ffma_peak(int device, double *tflops)
{
    if (!tflops) return fail(GI_ERR_INVALID_ARG, "tflops is NULL");
    DeviceGuard g(device);
    cudaDeviceProp prop;
    GI_CUDA(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    const int blocks = prop.multiProcessorCount * 8, iters = 4096;
    float *sink = nullptr;
    cudaEvent_t e0, e1;
    GI_CUDA(cudaMalloc(&sink, blocks * sizeof(float)), "cudaMalloc sink");
    GI_CUDA(cudaEventCreate(&e0), "cudaEventCreate");
    GI_CUDA(cudaEventCreate(&e1), "cudaEventCreate");
    float best = 1e30f;
    for (int rep = 0; rep < 8; ++rep) {
        cudaEventRecord(e0, 0);
        cudaError_t e = gi_launch_ffma_peak(sink, blocks, iters, 0);
        cudaEventRecord(e1, 0);
        if (e != cudaSuccess) { cudaFree(sink); return cuda_fail(e, "ffma kernel"); }
        GI_CUDA(cudaEventSynchronize(e1), "cudaEventSynchronize");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep >= 2) best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    const double flops = 2.0 * 8 * 16 * (double)iters * 256.0 * blocks;
    *tflops = flops / (best * 1e-3) / 1e12;
    return GI_OK;
}

// -------------------------------------------------------- drop-in wrappers --

static std::mutex g_default_mutex;
static gi_ctx *g_default_ctx[64] = {nullptr};

static int default_ctx(gi_ctx **out)
{
    int d = 0;
    GI_CUDA(cudaGetDevice(&d), "cudaGetDevice");
    if (d < 0 || d >= 64) return fail(GI_ERR_NO_DEVICE, "device %d", d);
    std::lock_guard<std::mutex> lk(g_default_mutex);
    if (!g_default_ctx[d]) {
        gi_ctx *c = nullptr;
        int st = gi_ctx_create(&c, d);
        if (st) return st;
        g_default_ctx[d] = c;
    }
    *out = g_default_ctx[d];
    return GI_OK;
}

extern "C" int gi_forces_collision(const float *pos, const float *vel, float *force,
                                   const gi_force_collision_consts *cc, int n, void *stream)
{
    if (!cc) return fail(GI_ERR_INVALID_ARG, "consts is NULL");
    if (n < 0) return fail(GI_ERR_BAD_SIZE, "n = %d", n);
    if (cc->NFe < 0) return fail(GI_ERR_BAD_SIZE, "NFe = %d", cc->NFe);
    if (n == 0) return GI_OK;
    gi_ctx *c = nullptr;
    int st = default_ctx(&c);
    if (st) return st;
    gi_pair_params p;
    gi_params_from_collision_consts(cc, &p);
    gi_run r{0, n, std::min(cc->NFe, n), 0, 0.0f, 0.0f, 0.0f, 0.0f};
    std::lock_guard<std::mutex> lk(g_default_mutex);
    return gi_forces(c, pos, vel, force, &r, 1, &p, 1, stream);
}

extern "C" int gi_move_collision(float *pos, float *vel, const float *force,
                                 const gi_move_collision_consts *mc, int n, void *stream)
{
    if (!mc) return fail(GI_ERR_INVALID_ARG, "consts is NULL");
    if (n < 0) return fail(GI_ERR_BAD_SIZE, "n = %d", n);
    if (mc->NFe < 0) return fail(GI_ERR_BAD_SIZE, "NFe = %d", mc->NFe);
    if (n == 0) return GI_OK;
    gi_run r{0, n, std::min(mc->NFe, n), 0, mc->Dt, mc->DtOverMassFe, mc->DtOverMassSi, 0.0f};
    return move_impl(pos, vel, force, &r, 1, (cudaStream_t)stream);
}

static int separate_runs(int b1, int b2, int b3, int n, gi_run r[2])
{
    if (n < 0) return fail(GI_ERR_BAD_SIZE, "n = %d", n);
    if (!(0 <= b1 && b1 <= b2 && b2 <= b3 && b3 <= n))
        return fail(GI_ERR_BAD_SIZE, "need 0 <= boarder1 <= boarder2 <= boarder3 <= n (%d %d %d %d)",
                    b1, b2, b3, n);
    r[0] = gi_run{0, b2, b1, 0, 0.0f, 0.0f, 0.0f, 0.0f};
    r[1] = gi_run{b2, n - b2, b3 - b2, 0, 0.0f, 0.0f, 0.0f, 0.0f};
    return GI_OK;
}

extern "C" int gi_params_from_separate_consts(const gi_force_separate_consts *c,
                                              gi_pair_params *out)
{
    if (!c || !out) return fail(GI_ERR_INVALID_ARG, "NULL argument");
    separate_params(c, out);
    return GI_OK;
}

extern "C" int gi_forces_separate(const float *pos, const float *vel, float *force,
                                  const gi_force_separate_consts *sc, int n, void *stream)
{
    if (!sc) return fail(GI_ERR_INVALID_ARG, "consts is NULL");
    gi_run r[2];
    int st = separate_runs(sc->boarder1, sc->boarder2, sc->boarder3, n, r);
    if (st) return st;
    if (n == 0) return GI_OK;
    gi_ctx *c = nullptr;
    if ((st = default_ctx(&c))) return st;
    gi_pair_params p;
    separate_params(sc, &p);
    std::lock_guard<std::mutex> lk(g_default_mutex);
    return gi_forces(c, pos, vel, force, r, 2, &p, 1, stream);
}

extern "C" int gi_move_damped_separate(float *pos, float *vel, const float *force,
                                       const gi_move_separate_consts *mc, float damp1,
                                       float damp2, int n, void *stream)
{
    if (!mc) return fail(GI_ERR_INVALID_ARG, "consts is NULL");
    gi_run r[2];
    int st = separate_runs(mc->boarder1, mc->boarder2, mc->boarder3, n, r);
    if (st) return st;
    if (n == 0) return GI_OK;
    for (int k = 0; k < 2; ++k) {
        r[k].dt = mc->Dt;
        r[k].dt_over_mass_fe = mc->DtOverMassFe;
        r[k].dt_over_mass_si = mc->DtOverMassSi;
    }
    r[0].damp = damp1;
    r[1].damp = damp2;
    return move_impl(pos, vel, force, r, 2, (cudaStream_t)stream);
}

// ---------------------------------------------------- graph-captured loops --

struct gi_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int device = 0;
};

extern "C" int gi_graph_create(gi_ctx *c, float *pos_a, float *vel_a, float *pos_b, float *vel_b,
                               const gi_run *runs, int nruns, const gi_pair_params *params,
                               int nparams, int nsteps, void *stream, gi_graph **out)
{
    if (!c || !out) return fail(GI_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (nsteps < 1) return fail(GI_ERR_INVALID_ARG, "nsteps = %d", nsteps);
    cudaStream_t s = (cudaStream_t)stream;
    if (s == nullptr)
        return fail(GI_ERR_INVALID_ARG, "capture needs a non-default stream");
    DeviceGuard g(c->device);
    // One uncaptured step sizes every scratch buffer (capture cannot allocate);
    // it steps a -> b, so the caller's state must be re-read from a: it is,
    // because the captured loop reads a first and the step above never wrote a.
    int st = gi_step_pingpong(c, pos_a, vel_a, pos_b, vel_b, runs, nruns, params, nparams, 1, stream);
    if (st) return st;
    GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    GI_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    st = gi_step_pingpong(c, pos_a, vel_a, pos_b, vel_b, runs, nruns, params, nparams, nsteps, stream);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (st) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return cuda_fail(e, "cudaGraphInstantiate");
    }
    gi_graph *gr = new gi_graph();
    gr->graph = graph;
    gr->exec = exec;
    gr->device = c->device;
    *out = gr;
    return GI_OK;
}

extern "C" int gi_graph_launch(gi_graph *gr, void *stream)
{
    if (!gr) return fail(GI_ERR_INVALID_ARG, "graph is NULL");
    DeviceGuard g(gr->device);
    GI_CUDA(cudaGraphLaunch(gr->exec, (cudaStream_t)stream), "cudaGraphLaunch");
    return GI_OK;
}

extern "C" int gi_graph_destroy(gi_graph *gr)
{
    if (!gr) return GI_OK;
    DeviceGuard g(gr->device);
    cudaGraphExecDestroy(gr->exec);
    cudaGraphDestroy(gr->graph);
    delete gr;
    return GI_OK;
}

// ------------------------------------------------------ internal helpers --

int gi_internal_fail(int status, const char *msg) { return fail(status, "%s", msg); }

int gi_internal_ctx_device(gi_ctx *c) { return c ? c->device : -1; }

int gi_internal_ctx_cluster_tries(gi_ctx *c)
{
    return (c && c->opt.cluster_tries > 0) ? c->opt.cluster_tries : (1 << 22);
}

int gi_internal_collision_pairdev(const gi_force_collision_consts *c, PairDev *d)
{
    gi_pair_params p;
    gi_params_from_collision_consts(c, &p);
    return to_device_params(p, *d);
}

// Device bytes of scratch one run of n bodies needs in this context (split-j
// partials, contact corrections, grid): the serving loop's admission estimate.
long long gi_internal_scratch_bytes(gi_ctx *c, int n)
{
    if (n <= 0) return 0;
    // far-field sums (3 x 8 bytes a body), contact corrections and the grid
    const long long common = 24LL * n + 24LL * n + 4LL * (long long)gi_grid_words(n, n);
    if (c->opt.accum == GI_ACC_PAIRED) return common;
    int ipt = 1, jc = GI_NT, lg = 0, tiles = 0, nsplit = 1;
    tuning_for(c, n, &ipt, &jc);
    chunking(n, jc, &lg, &tiles, &nsplit);
    const long long partials = nsplit > 1 ? (long long)nsplit * 3 * 8 * n : 0;
    const long long tickets = 4LL * ((n + GI_NT - 1) / GI_NT);
    return partials + common + tickets;
}
