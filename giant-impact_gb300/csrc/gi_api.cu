// gi_api.cu -- the C ABI of libgi.so: argument checking, the work-decomposition
// planner, context-owned scratch memory and the entry points declared in
// include/gi_api.h.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gi_internal.h"

int gi_force_occupancy_ipt1(int acc, int epi);
int gi_force_occupancy_ipt2(int acc, int epi);
int gi_force_occupancy_ipt4(int acc, int epi);

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
                            const LaunchTable &tab, cudaStream_t s)
{
    switch (ipt) {
    case 1: return gi_launch_force_ipt1(acc, epi, a, tab, s);
    case 2: return gi_launch_force_ipt2(acc, epi, a, tab, s);
    case 4: return gi_launch_force_ipt4(acc, epi, a, tab, s);
    default: return cudaErrorInvalidValue;
    }
}

int gi_force_occupancy(int ipt, int acc, int epi)
{
    switch (ipt) {
    case 1: return gi_force_occupancy_ipt1(acc, epi);
    case 2: return gi_force_occupancy_ipt2(acc, epi);
    case 4: return gi_force_occupancy_ipt4(acc, epi);
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
    if (p.GMassFeFe < 0.0f || p.GMassSiSi < 0.0f || p.GMassFeSi < 0.0f)
        return fail(GI_ERR_PARAMS, "negative G*m*m in the pair table");
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

struct gi_ctx {
    int device = 0;
    int sm_count = 0;
    gi_options opt{GI_SEP_REF_INT, GI_ACCUM_KAHAN};
    bool forced = false;
    gi_tuning forced_tuning{0, 0};
    // Tuned decomposition per N bucket (floor(log2 n)): i-bodies per thread
    // and the number of work items a run is split into.
    int bucket_ipt[32] = {0};
    int bucket_items[32] = {0};
    unsigned int *tickets = nullptr;
    size_t tickets_cap = 0;
    double *partials = nullptr;
    size_t partials_cap = 0;  // doubles
    float4 *pp_pos = nullptr, *pp_vel = nullptr;
    size_t pp_cap = 0;  // bodies
    float4 *mirror_pos = nullptr, *mirror_vel = nullptr;
    size_t mirror_cap = 0;
    double *diag_work = nullptr;  // 16 doubles per block + 16 for the result
    int diag_blocks = 0;
    double *pot_buf = nullptr;
    size_t pot_cap = 0;
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
    c->diag_blocks = 2 * c->sm_count;
    return GI_OK;
}

static void ctx_free(gi_ctx *c)
{
    DeviceGuard g(c->device);
    cudaFree(c->tickets);
    cudaFree(c->partials);
    cudaFree(c->pp_pos);
    cudaFree(c->pp_vel);
    cudaFree(c->mirror_pos);
    cudaFree(c->mirror_vel);
    cudaFree(c->diag_work);
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
    if (o->accum < GI_ACCUM_KAHAN || o->accum > GI_ACCUM_FP64)
        return fail(GI_ERR_INVALID_ARG, "accum %d", o->accum);
    c->opt = *o;
    return GI_OK;
}

extern "C" int gi_ctx_set_tuning(gi_ctx *c, const gi_tuning *t)
{
    if (!c) return fail(GI_ERR_INVALID_ARG, "ctx is NULL");
    if (!t) { c->forced = false; return GI_OK; }
    if (t->i_per_thread != 1 && t->i_per_thread != 2 && t->i_per_thread != 4)
        return fail(GI_ERR_INVALID_ARG, "i_per_thread must be 1, 2 or 4");
    if (t->jchunk < 0 || t->jchunk % GI_NT != 0)
        return fail(GI_ERR_INVALID_ARG, "jchunk must be a non-negative multiple of %d", GI_NT);
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
        *jchunk = jc;
        return;
    }
    const int b = bucket_of(std::max(n, 1));
    int p = c->bucket_ipt[b];
    int items = c->bucket_items[b];
    if (p == 0) {
        p = n >= 32768 ? 4 : (n >= 8192 ? 2 : 1);
        items = 16 * c->sm_count;
    }
    const int ib = GI_NT * p;
    const int nib = (n + ib - 1) / ib;
    int nsplit = std::max(1, (items + nib - 1) / std::max(nib, 1));
    nsplit = std::min(nsplit, std::max(1, n / 1024));
    int jc = (n + nsplit - 1) / nsplit;
    jc = ((jc + GI_NT - 1) / GI_NT) * GI_NT;
    *ipt = p;
    *jchunk = std::max(jc, GI_NT);
}

extern "C" int gi_ctx_get_tuning(gi_ctx *c, int n, gi_tuning *out)
{
    if (!c || !out) return fail(GI_ERR_INVALID_ARG, "NULL argument");
    if (n < 0) return fail(GI_ERR_BAD_SIZE, "n = %d", n);
    tuning_for(c, n, &out->i_per_thread, &out->jchunk);
    return GI_OK;
}

// ---------------------------------------------------------------- planning --

struct Plan {
    std::vector<LaunchTable> tables;
    std::vector<int> ipt;
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

static int make_plan(const gi_ctx *c, const gi_run *runs, int nruns,
                     const std::vector<PairDev> &pd, Plan &plan)
{
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
        const int p = ipt[order[k]];
        long long items = 0, tick = 0, part = 0;
        while (k < order.size() && ipt[order[k]] == p && t.nruns < GI_MAX_RUNS) {
            const gi_run &q = runs[order[k]];
            RunDev &d = t.runs[t.nruns++];
            d.offset = q.offset;
            d.n = q.n;
            d.nfe = q.nfe;
            d.param = q.params;
            d.jchunk = jc[order[k]];
            d.nsplit = (q.n + d.jchunk - 1) / d.jchunk;
            d.nib = (q.n + GI_NT * p - 1) / (GI_NT * p);
            d.ipt = p;
            d.item_start = (int)items;
            items += (long long)d.nib * d.nsplit;
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

static int ensure_scratch(gi_ctx *c, const Plan &plan, cudaStream_t s)
{
    const bool grow_t = plan.tickets > c->tickets_cap;
    const bool grow_p = plan.partials > c->partials_cap;
    if (!grow_t && !grow_p) return GI_OK;
    if (stream_capturing(s))
        return fail(GI_ERR_INVALID_ARG,
                    "scratch must grow (run once outside stream capture before capturing)");
    GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (grow_t) {
        cudaFree(c->tickets);
        c->tickets = nullptr;
        c->tickets_cap = 0;
        size_t cap = std::max(plan.tickets, (size_t)1024);
        GI_CUDA(cudaMalloc(&c->tickets, cap * sizeof(unsigned int)), "cudaMalloc tickets");
        GI_CUDA(cudaMemset(c->tickets, 0, cap * sizeof(unsigned int)), "cudaMemset tickets");
        c->tickets_cap = cap;
    }
    if (grow_p) {
        cudaFree(c->partials);
        c->partials = nullptr;
        c->partials_cap = 0;
        size_t cap = plan.partials + plan.partials / 4;
        GI_CUDA(cudaMalloc(&c->partials, cap * sizeof(double)), "cudaMalloc partials");
        c->partials_cap = cap;
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

static int run_force_plan(gi_ctx *c, const Plan &plan, int epi, const float4 *pos,
                          const float4 *vel, float4 *force, float4 *pos_out,
                          float4 *vel_out, cudaStream_t s)
{
    for (size_t t = 0; t < plan.tables.size(); ++t) {
        ForceArgs a;
        a.pos = pos;
        a.vel = vel;
        a.force = force;
        a.pos_out = pos_out;
        a.vel_out = vel_out;
        a.partials = c->partials;
        a.tickets = c->tickets;
        GI_CUDA(gi_launch_force(plan.ipt[t], c->opt.accum, epi, a, plan.tables[t], s),
                "force kernel launch");
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
    if ((st = ensure_scratch(c, plan, s))) return st;
    return run_force_plan(c, plan, GI_EPI_FORCE, (const float4 *)pos, (const float4 *)vel,
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

static int ensure_pingpong(gi_ctx *c, size_t bodies, cudaStream_t s)
{
    if (bodies <= c->pp_cap) return GI_OK;
    if (stream_capturing(s))
        return fail(GI_ERR_INVALID_ARG,
                    "state buffers must grow (run once outside stream capture before capturing)");
    GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    cudaFree(c->pp_pos);
    cudaFree(c->pp_vel);
    c->pp_pos = c->pp_vel = nullptr;
    c->pp_cap = 0;
    GI_CUDA(cudaMalloc(&c->pp_pos, bodies * sizeof(float4)), "cudaMalloc state");
    GI_CUDA(cudaMalloc(&c->pp_vel, bodies * sizeof(float4)), "cudaMalloc state");
    c->pp_cap = bodies;
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
    if ((st = ensure_scratch(c, plan, s))) return st;
    if ((st = ensure_pingpong(c, (size_t)plan.max_end, s))) return st;
    float4 *ip = (float4 *)pos, *iv = (float4 *)vel, *op = c->pp_pos, *ov = c->pp_vel;
    for (int k = 0; k < nsteps; ++k) {
        if ((st = run_force_plan(c, plan, GI_EPI_STEP, ip, iv, nullptr, op, ov, s))) return st;
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
        c->mirror_pos = c->mirror_vel = nullptr;
        c->mirror_cap = 0;
        GI_CUDA(cudaMalloc(&c->mirror_pos, ntotal * sizeof(float4)), "cudaMalloc mirror");
        GI_CUDA(cudaMalloc(&c->mirror_vel, ntotal * sizeof(float4)), "cudaMalloc mirror");
        c->mirror_cap = ntotal;
    }
    const size_t bytes = (size_t)ntotal * sizeof(float4);
    GI_CUDA(cudaMemcpyAsync(c->mirror_pos, pos_host, bytes, cudaMemcpyHostToDevice, s), "H2D pos");
    GI_CUDA(cudaMemcpyAsync(c->mirror_vel, vel_host, bytes, cudaMemcpyHostToDevice, s), "H2D vel");
    st = gi_step(c, (float *)c->mirror_pos, (float *)c->mirror_vel, runs, nruns, params,
                 nparams, nsteps, stream);
    if (st) return st;
    GI_CUDA(cudaMemcpyAsync(pos_host, c->mirror_pos, bytes, cudaMemcpyDeviceToHost, s), "D2H pos");
    GI_CUDA(cudaMemcpyAsync(vel_host, c->mirror_vel, bytes, cudaMemcpyDeviceToHost, s), "D2H vel");
    GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    return GI_OK;
}

extern "C" int gi_diag_fp64(gi_ctx *c, const float *pos, const float *vel,
                            const unsigned char *label, int scope, const gi_run *run,
                            const gi_pair_params *params, double *out, void *stream)
{
    if (!c || !run || !params || !out) return fail(GI_ERR_INVALID_ARG, "NULL argument");
    if (scope < 0 || scope > 3) return fail(GI_ERR_INVALID_ARG, "scope %d", scope);
    gi_run q = *run;
    q.params = 0;
    int st = check_runs(&q, 1, 1);
    if (st) return st;
    if ((st = check_body_ptr(pos, "pos")) || (st = check_body_ptr(vel, "vel"))) return st;
    DeviceGuard g(c->device);
    cudaStream_t s = (cudaStream_t)stream;
    if (!c->diag_work) {
        GI_CUDA(cudaMalloc(&c->diag_work, (size_t)(c->diag_blocks + 1) * 16 * sizeof(double)),
                "cudaMalloc diag");
    }
    double *out_dev = c->diag_work + (size_t)c->diag_blocks * 16;
    RunDev rd;
    std::memset(&rd, 0, sizeof rd);
    rd.offset = q.offset;
    rd.n = q.n;
    rd.nfe = q.nfe;
    PairDev pdv;
    std::memset(&pdv, 0, sizeof pdv);
    GI_CUDA(gi_launch_diag((const float4 *)pos, (const float4 *)vel, label, scope, rd, pdv,
                           params->MassFe, params->MassSi, c->diag_work, c->diag_blocks,
                           out_dev, s),
            "diag launch");
    GI_CUDA(cudaMemcpyAsync(out, out_dev, 15 * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H diag");
    GI_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
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
