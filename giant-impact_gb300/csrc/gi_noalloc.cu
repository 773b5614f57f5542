// gi_noalloc.cu -- the collision force pass for callers that cannot allocate
// device memory.
//
// gi_forces_collision, the regular drop-in, takes its scratch memory
// (far-field sums, cell grid, contact corrections) from a library context
// that grows it with cudaMalloc on first use.  Some callers
// cannot let a library do that:
//   - applications that hand out device memory only from their own budget or
//     pool (a run admitted against a fixed HBM budget, a GPU shared under a
//     per-process memory limit), where a hidden allocation could fail at an
//     arbitrary step or silently break the budget;
//   - latency-sensitive step loops that must not stall: cudaMalloc and
//     cudaFree can synchronise the whole device, holding up every stream.
// For them, gi_forces_collision_noalloc computes the same forces, bit for bit
// (the same kernels with the same default decomposition), with all of its
// scratch in one statically allocated device array, g_noalloc_scratch, of
// GI_NOALLOC_BYTES (8 MiB; the largest run takes 4.3 MiB of it).  Every GPU that loads the library holds that
// array until the process exits.  The array limits a call to
// GI_NOALLOC_MAX_BODIES (32,768) bodies; larger calls are refused.
//
// Every call shares the one array and leaves its contents behind: the
// far-field sums and the grid's counters, which must start at zero, are
// cleared at the start of each call (in stream order); everything else is
// fully written before it is read.  Calls
// that overlap on the GPU (for example on two streams) race on the array and
// corrupt each other's results; serialise them.
//
// Host code cannot use the array's name as a device address (on the host it
// names a stand-in object).  The device address is obtained once per device
// with cudaGetSymbolAddress, with that device current, by the first call on
// that device; make that first call before any stream capture.  The address
// is remembered together with the identity of the device's CUDA context, so
// after a cudaDeviceReset (a new context, where the array may lie elsewhere)
// the next call looks it up again; make that call outside capture too.
#include <cuda.h>

#include <cstring>
#include <mutex>

#include "gi_internal.h"

#define GI_NOALLOC_BYTES (8u << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[GI_NOALLOC_BYTES];

namespace {

constexpr size_t kMaxBodies = GI_NOALLOC_MAX_BODIES;
constexpr size_t kTriple = 3 * sizeof(long long);  // one int64 triple per body
constexpr size_t kSumOff = 0;                         // far-field sums (paired kernel)
constexpr size_t kDeltaOff = kSumOff + kTriple * kMaxBodies;  // contact corrections
constexpr size_t kGridOff = kDeltaOff + kTriple * kMaxBodies;  // the cell grid

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// The carve of the static array: far-field sums and contact corrections
// sized for the largest run, then the cell grid of this run.  The grid grows
// with n, so the largest run accepted is the one to check; it is checked
// here, at compile time, so that a change of the grid's layout cannot leave
// maximum-size calls refused.
constexpr size_t grid_end_for(size_t n)
{
    return kGridOff + align256(gi_grid_words((long long)n, (long long)n) * sizeof(unsigned int));
}
static_assert(grid_end_for(kMaxBodies) <= GI_NOALLOC_BYTES,
              "the static scratch does not hold the largest run");
static_assert(kDeltaOff % 256 == 0 && kGridOff % 256 == 0, "carve offsets must stay aligned");

std::mutex g_mu;
void *g_base[64] = {nullptr};
unsigned long long g_ctx_id[64] = {0};

// Identity of the calling thread's current CUDA context (0 if none is
// current or the driver does not say).  The driver calls are looked up
// through the runtime, so libgi does not link against the driver library.
unsigned long long current_context_id()
{
    typedef CUresult (*GetCurrent)(CUcontext *);
    typedef CUresult (*GetId)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        looked_up = true;
        void *f = nullptr, *g = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q1) ==
                cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &g, 12000, cudaEnableDefault, &q2) ==
                cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<GetCurrent>(f);
            get_id = reinterpret_cast<GetId>(g);
        }
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c) return 0;
    if (get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of g_noalloc_scratch on the current device: looked up on
// the first call per device, and again when the device's context is a new
// one (after a device reset).  With no context identity to go by it is
// looked up on every call.
int scratch_base(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return gi_internal_fail(GI_ERR_CUDA, "cudaGetDevice failed");
    if (dev < 0 || dev >= 64) return gi_internal_fail(GI_ERR_NO_DEVICE, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    const unsigned long long id = current_context_id();
    if (!g_base[dev] || id == 0 || id != g_ctx_id[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
        if (e != cudaSuccess)
            return gi_internal_fail(GI_ERR_CUDA, "cudaGetSymbolAddress of the static scratch failed");
        g_base[dev] = ptr;
        g_ctx_id[dev] = current_context_id();  // the lookup made the context current
    }
    *out = g_base[dev];
    return GI_OK;
}

}  // namespace

extern "C" int gi_forces_collision_noalloc(const float *pos, const float *vel, float *force,
                                           const gi_force_collision_consts *cc, int n,
                                           void *stream)
{
    if (!cc) return gi_internal_fail(GI_ERR_INVALID_ARG, "consts is NULL");
    if (n < 0) return gi_internal_fail(GI_ERR_BAD_SIZE, "n is negative");
    if ((size_t)n > kMaxBodies)
        return gi_internal_fail(GI_ERR_BAD_SIZE,
                                "gi_forces_collision_noalloc takes at most GI_NOALLOC_MAX_BODIES "
                                "(32768) bodies; use gi_forces_collision for larger runs");
    if (cc->NFe < 0) return gi_internal_fail(GI_ERR_BAD_SIZE, "NFe is negative");
    if (n == 0) return GI_OK;
    if (!pos || !vel || !force) return gi_internal_fail(GI_ERR_INVALID_ARG, "body array is NULL");
    if ((reinterpret_cast<uintptr_t>(pos) | reinterpret_cast<uintptr_t>(vel) |
         reinterpret_cast<uintptr_t>(force)) % 16 != 0)
        return gi_internal_fail(GI_ERR_ALIGNMENT, "body arrays must be 16-byte aligned");

    LaunchTable tab;
    std::memset(&tab, 0, sizeof tab);
    int st = gi_internal_collision_pairdev(cc, &tab.params[0]);
    if (st) return st;
    RunDev &d = tab.runs[0];
    d.offset = 0;
    d.n = n;
    d.nfe = cc->NFe < n ? cc->NFe : n;
    d.param = 0;
    // The default decomposition of gi_forces_collision's context, so both
    // entry points give the same bits.
    const long long items = gi_internal_pair_run(d, n, gi_internal_pair_default_pcl(n),
                                                 tab.params[0], 0);
    tab.nruns = 1;
    tab.nitems = (int)items;
    tab.sep_test = GI_SEP_REF_INT;
    tab.dense_min = 256;

    // Carve the static array (the largest run is checked to fit at compile
    // time; this guards the arithmetic at run time as well).
    if (grid_end_for((size_t)n) > GI_NOALLOC_BYTES)
        return gi_internal_fail(GI_ERR_BAD_SIZE, "static scratch layout does not fit this run");
    void *base = nullptr;
    if ((st = scratch_base(&base))) return st;
    unsigned char *b = static_cast<unsigned char *>(base);
    long long *sums = reinterpret_cast<long long *>(b + kSumOff);
    long long *delta = reinterpret_cast<long long *>(b + kDeltaOff);
    unsigned int *grid = reinterpret_cast<unsigned int *>(b + kGridOff);

    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return gi_internal_fail(GI_ERR_CUDA, "device query failed");
    cudaStream_t s = (cudaStream_t)stream;
    // The far-field sums must start at zero; the array keeps whatever the
    // previous call left, so clear them in stream order.
    if (cudaMemsetAsync(sums, 0, kTriple * (size_t)n, s) != cudaSuccess)
        return gi_internal_fail(GI_ERR_CUDA, "clearing the static scratch sums failed");
    if (gi_launch_contacts(reinterpret_cast<const float4 *>(pos), reinterpret_cast<const float4 *>(vel),
                           tab, n, n, grid, delta, nsm, s) != cudaSuccess)
        return gi_internal_fail(GI_ERR_CUDA, "contact pass launch failed");
    ForceArgs a;
    std::memset(&a, 0, sizeof a);
    a.pos = reinterpret_cast<const float4 *>(pos);
    a.vel = reinterpret_cast<const float4 *>(vel);
    a.force = reinterpret_cast<float4 *>(force);
    a.delta = delta;
    a.fsum_fx = sums;
    if (gi_launch_pair_force(a, tab, s) != cudaSuccess)
        return gi_internal_fail(GI_ERR_CUDA, "force kernel launch failed");
    if (gi_launch_pair_finish(GI_EPI_FORCE, a, tab, n, nsm, s) != cudaSuccess)
        return gi_internal_fail(GI_ERR_CUDA, "epilogue launch failed");
    return GI_OK;
}
