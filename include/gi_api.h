/*
 * gi_api.h -- C ABI of the GB300 (sm_103a) Giant-Impact force / kick-drift
 * library, libgi.so.
 *
 * Conventions
 *   - Body arrays are float4 arrays passed as `float *` (4 floats per body,
 *     16-byte aligned): pos = (x, y, z, tag), vel = (vx, vy, vz, mass),
 *     force = (fx, fy, fz, unused).  Kernels write only .xyz and leave .w
 *     as it was, like the reference kernels.
 *   - Material is given by index, as in the reference: within a body set
 *     ("run") the first nfe bodies are Fe, the rest Si.
 *   - Device pointers unless a function says otherwise.  `stream` is a
 *     cudaStream_t passed as void* (NULL = legacy default stream, which is
 *     what the reference launches on).  Every call is stream-ordered and
 *     asynchronous unless documented otherwise.
 *   - Every entry point returns a gi_status (0 = GI_OK).  Nothing calls
 *     exit(); gi_last_error() holds a message for the calling thread.
 *
 * Reference interfaces replaced (paths relative to the Giant-Impact
 * project) are cited beside each entry point.
 */
#ifndef GI_API_H
#define GI_API_H

#ifdef __cplusplus
extern "C" {
#endif

#define GI_API_VERSION 1

typedef enum gi_status {
    GI_OK = 0,
    GI_ERR_INVALID_ARG = 1,  /* null pointer, negative count, unknown enum   */
    GI_ERR_BAD_SIZE = 2,     /* n or nfe out of range, table too large       */
    GI_ERR_ALIGNMENT = 3,    /* body array not 16-byte aligned               */
    GI_ERR_CUDA = 4,         /* CUDA runtime error (message in last_error)   */
    GI_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up           */
    GI_ERR_NO_DEVICE = 6,    /* no CUDA device / sm_103 kernels unavailable  */
    GI_ERR_OUT_OF_MEMORY = 7,
    GI_ERR_PARAMS = 8,       /* inconsistent physical parameters             */
    GI_ERR_IO = 9,           /* file could not be opened / read / written    */
    GI_ERR_FORMAT = 10,      /* file contents malformed or truncated         */
    GI_ERR_CAPACITY = 11     /* admission refused: memory budget or slots    */
} gi_status;

/* ------------------------------------------------------------------------ */
/* Reference-layout constant structures                                     */
/* ------------------------------------------------------------------------ */

/* Layout-identical to forceCollisionKernalConstantsStruct
 * (Code/ImpactCode/impactAddTime.cu:4-20).  The reference hard-codes the
 * Si-Si gravity G*mSi*mSi as 1 (impactAddTime.cu:302); the drop-in entry
 * points keep that convention. */
typedef struct gi_force_collision_consts {
    float GMassFeFe;
    float GMassFeSi;
    float KFeFe;
    float KSiSi;
    float KFeSi;
    float KRFeFe;
    float KRSiSi;
    float KRFeSi;
    float KRMix;
    float ShellBreakFe;
    float ShellBreakSi;
    float ShellBreakFeSi1;
    float ShellBreakFeSi2;
    int NFe;
} gi_force_collision_consts;

/* Layout-identical to moveCollisionKernalConstantsStruct
 * (Code/ImpactCode/impactAddTime.cu:22-28). */
typedef struct gi_move_collision_consts {
    float Dt;
    float DtOverMassFe;
    float DtOverMassSi;
    int NFe;
} gi_move_collision_consts;

/* Layout-identical to forceSeperateKernalConstantsStruct
 * (Code/GenerateTargetImpactorCode/generateTargetImpactor.cu:3-21).
 * Bodies are ordered [Fe1, Si1, Fe2, Si2]: boarder1 = end of Fe1,
 * boarder2 = end of body 1, boarder3 = end of Fe2. */
typedef struct gi_force_separate_consts {
    float GMassFeFe;
    float GMassFeSi;
    float KFeFe;
    float KSiSi;
    float KFeSi;
    float KRFeFe;
    float KRSiSi;
    float KRFeSi;
    float KRMix;
    float ShellBreakFe;
    float ShellBreakSi;
    float ShellBreakFeSi1;
    float ShellBreakFeSi2;
    int boarder1;
    int boarder2;
    int boarder3;
} gi_force_separate_consts;

/* Layout-identical to moveSeperateKernalConstantsStruct
 * (Code/GenerateTargetImpactorCode/generateTargetImpactor.cu:23-31). */
typedef struct gi_move_separate_consts {
    float Dt;
    float DtOverMassFe;
    float DtOverMassSi;
    int boarder1;
    int boarder2;
    int boarder3;
} gi_move_separate_consts;

/* ------------------------------------------------------------------------ */
/* General (multi-run) description                                          */
/* ------------------------------------------------------------------------ */

/* Pair table of one material set.  GMass* = G m_i m_j per pair class,
 * K* = pair stiffness (KFeFe = 2 KFe, KFeSi = KFe + KSi, ...), KR* = the
 * reduced stiffness of a separating pair inside its shell, ShellBreak* =
 * D (1 - SD) (impactAddTime.cu:128-170).  MassFe / MassSi are the element
 * masses (used by the FP64 diagnostics).  The gravity table must be
 * positive and rank one: GMassFeSi^2 == GMassFeFe * GMassSiSi (true
 * whenever it comes from G > 0, mFe, mSi). */
typedef struct gi_pair_params {
    float GMassFeFe, GMassFeSi, GMassSiSi;
    float KFeFe, KSiSi, KFeSi;
    float KRFeFe, KRSiSi, KRFeSi, KRMix;
    float ShellBreakFe, ShellBreakSi, ShellBreakFeSi1, ShellBreakFeSi2;
    float MassFe, MassSi;
} gi_pair_params;

/* One independent body set.  Bodies [offset, offset + n) interact only
 * with each other; [offset, offset + nfe) are Fe.  Kick-drift constants:
 * v += (F - damp v) * dt_over_mass; x += v dt. */
typedef struct gi_run {
    int offset;
    int n;
    int nfe;
    int params;            /* index into the gi_pair_params table */
    float dt;
    float dt_over_mass_fe;
    float dt_over_mass_si;
    float damp;
} gi_run;

/* Separation test (which contact pairs use the reduced KR). */
#define GI_SEP_REF_INT 0   /* reference: int inout = dp.dv; KR if inout > 0 */
#define GI_SEP_SIGN 1      /* KR if dp.dv > 0                               */

/* Per-body force accumulation. */
#define GI_ACCUM_KAHAN 0   /* FP32 per j-tile, Kahan-compensated across tiles */
#define GI_ACCUM_FP32 1    /* FP32 per j-tile, plain FP32 across tiles        */
#define GI_ACCUM_FP64 2    /* FP32 per j-tile, FP64 across tiles              */

typedef struct gi_options {
    int sep_test;          /* GI_SEP_*, default GI_SEP_REF_INT */
    int accum;             /* GI_ACCUM_*, default GI_ACCUM_KAHAN */
} gi_options;

/* Work decomposition of one run (chosen per N bucket by the autotuner or
 * set explicitly).  i_per_thread in {1, 2, 4, 8}; jchunk = 128 * 2^k bodies
 * per big j-chunk (the last chunks shrink by halves to 128 bodies), or 0 =
 * the whole run in one chunk.  The result for a run depends only on these
 * two numbers, never on what else is in the batch. */
typedef struct gi_tuning {
    int i_per_thread;
    int jchunk;
} gi_tuning;

typedef struct gi_ctx gi_ctx;

/* ------------------------------------------------------------------------ */
/* Library                                                                  */
/* ------------------------------------------------------------------------ */

int gi_version(void);
const char *gi_status_string(int status);
/* Message of the last failed call on this host thread ("" if none). */
const char *gi_last_error(void);

/* Device facts used by the tuner and by bench.py (host call, synchronous). */
int gi_device_info(int device, int *sm_count, int *cc_major, int *cc_minor,
                   long long *global_mem_bytes);

/* ------------------------------------------------------------------------ */
/* Drop-in entry points (reference signatures, stateless)                   */
/* ------------------------------------------------------------------------ */

/* Replaces getForcesCollisionSingleGPU<<<N/256, 256>>>(Pos, Vel, Force, c)
 * (Code/ImpactCode/impactAddTime.cu:245-377, launched at :400).  Any n >= 0
 * (the reference needs n % 256 == 0).  Reference separation test, Kahan
 * accumulation.  Uses library-owned scratch on the current device. */
int gi_forces_collision(const float *pos, const float *vel, float *force,
                        const gi_force_collision_consts *c, int n, void *stream);

/* Replaces moveBodiesCollisionSingleGPU (impactAddTime.cu:379-394, :401). */
int gi_move_collision(float *pos, float *vel, const float *force,
                      const gi_move_collision_consts *c, int n, void *stream);

/* Replaces getForcesSeperate
 * (Code/GenerateTargetImpactorCode/generateTargetImpactor.cu:486-626,
 * launched at :670): two bodies, cross-body pairs skipped.  Si-Si gravity
 * is 1, as in the reference. */
int gi_forces_separate(const float *pos, const float *vel, float *force,
                       const gi_force_separate_consts *c, int n, void *stream);

/* Replaces moveBodiesDampedSeperate (generateTargetImpactor.cu:628-664,
 * launched at :684, :696, :711). */
int gi_move_damped_separate(float *pos, float *vel, const float *force,
                            const gi_move_separate_consts *c, float damp1,
                            float damp2, int n, void *stream);

/* Same force pass as gi_forces_collision for callers that cannot allocate
 * device memory: applications that hand out device memory only from their
 * own budget or pool (where a hidden cudaMalloc could fail mid-run or break
 * the budget), and step loops that must not stall on the device-wide
 * synchronisation cudaMalloc / cudaFree can cause.  It has no counterpart in
 * the reference, which allocates nothing beyond its three body arrays.
 * All scratch lives in one static device array of 10 MiB that every GPU
 * loading the library holds until exit, so a call takes at most
 * GI_NOALLOC_MAX_BODIES bodies (larger n returns GI_ERR_BAD_SIZE).  The
 * first call on a device looks the array up (cudaGetSymbolAddress); make it
 * before any stream capture.  Calls share the array: calls that overlap on
 * the GPU (e.g. on two streams) race, so serialise them.  Forces agree with
 * gi_forces_collision within the library's 1e-5 force tolerance (the
 * decomposition, hence the summation order, differs). */
#define GI_NOALLOC_MAX_BODIES 32768
int gi_forces_collision_noalloc(const float *pos, const float *vel, float *force,
                                const gi_force_collision_consts *c, int n, void *stream);

/* ------------------------------------------------------------------------ */
/* Context API (multi-run, fused step, diagnostics)                         */
/* ------------------------------------------------------------------------ */

/* A context owns scratch memory (split-j partial sums, ping-pong state),
 * options and the tuning table for one device.  Not thread-safe: use one
 * context per host thread.  Allocates lazily, on first use. */
int gi_ctx_create(gi_ctx **ctx, int device);
int gi_ctx_destroy(gi_ctx *ctx);
int gi_ctx_set_options(gi_ctx *ctx, const gi_options *opt);
/* Force a decomposition for every run (NULL = back to the tuned table). */
int gi_ctx_set_tuning(gi_ctx *ctx, const gi_tuning *tuning);
/* The decomposition the context would use for a run of n bodies. */
int gi_ctx_get_tuning(gi_ctx *ctx, int n, gi_tuning *out);

/* Autotuner: for each N bucket (floor(log2 n)) among `runs`, times the
 * force pass for i_per_thread in {1, 2, 4} and five big-chunk sizes on the
 * caller's own bodies, and stores the fastest in the context (synchronous;
 * allocates a temporary force array).  Later calls decompose runs of those
 * buckets with the tuned values; results depend only on n and this table. */
int gi_autotune(gi_ctx *ctx, const float *pos, const float *vel, const gi_run *runs,
                int nruns, const gi_pair_params *params, int nparams, void *stream);

/* Force pass over nruns independent runs (one launch): force[i].xyz for
 * every body of every run. */
int gi_forces(gi_ctx *ctx, const float *pos, const float *vel, float *force,
              const gi_run *runs, int nruns, const gi_pair_params *params,
              int nparams, void *stream);

/* Kick-drift of every run with its own damp (v += (F - damp v) dt/m). */
int gi_move(gi_ctx *ctx, float *pos, float *vel, const float *force,
            const gi_run *runs, int nruns, void *stream);

/* nsteps fused force + kick-drift steps of every run, in place: one kernel
 * per step, reading one state buffer and writing the other (the context
 * owns the second buffer), so no force array round-trips through HBM.
 * Equivalent to nsteps x (gi_forces; gi_move). */
int gi_step(gi_ctx *ctx, float *pos, float *vel, const gi_run *runs,
            int nruns, const gi_pair_params *params, int nparams, int nsteps,
            void *stream);

/* nsteps fused steps alternating between two caller-owned state buffers
 * (a -> b -> a ...): the state after an odd number of steps is in b, after
 * an even number in a.  No copies, no library-owned state buffer: the
 * building block of graph-captured step loops.  Same kernels and results as
 * gi_step. */
int gi_step_pingpong(gi_ctx *ctx, float *pos_a, float *vel_a, float *pos_b,
                     float *vel_b, const gi_run *runs, int nruns,
                     const gi_pair_params *params, int nparams, int nsteps,
                     void *stream);

/* Graph-captured step loop: captures nsteps fused steps of the given runs
 * (gi_step_pingpong a -> b -> a ...) on `stream` (a non-default stream)
 * into a CUDA graph; each gi_graph_launch then advances every run nsteps
 * steps with one launch call.  Runs one uncaptured step first (a -> b) to
 * size the scratch memory, which capture cannot allocate; the captured loop
 * starts again from a.  The graph bakes in the buffers, runs and
 * decomposition: rebuild it when they change.  After a launch the state is
 * in b if nsteps is odd, in a if even. */
typedef struct gi_graph gi_graph;
int gi_graph_create(gi_ctx *ctx, float *pos_a, float *vel_a, float *pos_b, float *vel_b,
                    const gi_run *runs, int nruns, const gi_pair_params *params, int nparams,
                    int nsteps, void *stream, gi_graph **out);
int gi_graph_launch(gi_graph *graph, void *stream);
int gi_graph_destroy(gi_graph *graph);

/* FP64 diagnostics of one run (synchronous: returns with out filled).
 * label (device, one byte per body of the whole array, may be NULL)
 * selects scope: 0 = all, 1 = label 1 or 2 (Earth + Moon), 2 = label 1
 * (Earth), 3 = label 2 (Moon)  (impactBasicFunctions.h:219-652).
 * out[0..14] = mass, com xyz, com velocity xyz, angular momentum about the
 * com relative to the com velocity xyz, kinetic energy, momentum xyz,
 * body count. */
int gi_diag_fp64(gi_ctx *ctx, const float *pos, const float *vel,
                 const unsigned char *label, int scope, const gi_run *run,
                 const gi_pair_params *params, double *out, void *stream);

/* Pair potential energy of each run in FP64 (synchronous):
 * out[r] = 1/2 sum_i sum_{j != i} U(r_ij) with U = -G m m / r for r >= 1 and
 * -Gmm + Gmm (r - 1) - K (r - r^3/3 - 2/3) for r < 1 (the potential of the
 * full-K law; the reference computes no energy). */
int gi_potential_fp64(gi_ctx *ctx, const float *pos, const gi_run *runs,
                      int nruns, const gi_pair_params *params, int nparams,
                      double *out, void *stream);

/* End-to-end call with HOST buffers: copies pos/vel (pinned or pageable) to
 * the device, runs nsteps fused steps, copies them back, synchronises.
 * What a driver does between two records (impactAddTime.cu:396-431). */
int gi_run_host(gi_ctx *ctx, float *pos_host, float *vel_host, int ntotal,
                const gi_run *runs, int nruns, const gi_pair_params *params,
                int nparams, int nsteps, void *stream);

/* Measured FP32 FFMA throughput of the device in TFLOP/s (synchronous, a
 * ~50 ms microbenchmark): the denominator of the force kernel's roofline. */
int gi_measure_ffma_peak(int device, double *tflops);

/* ------------------------------------------------------------------------ */
/* Serving loop (continuous batching of impact runs)                        */
/* ------------------------------------------------------------------------ */

/* Requests wait in a FIFO queue.  Each gi_server_round admits queued runs
 * while a slot is free and their device memory (two state buffers plus the
 * scratch estimate) fits in the HBM budget, advances every live run
 * steps_per_round steps -- all live runs in one force launch per step --
 * and retires finished runs to host memory.  A run's result is the same
 * alone and in any mix (the force pass is batch-invariant).  The reference
 * runs one impact per process; this has no counterpart there. */
#define GI_SERVER_DRY_RUN (-1)   /* device value: schedule without a GPU */
#define GI_REQ_QUEUED 0
#define GI_REQ_LIVE 1
#define GI_REQ_DONE 2

typedef struct gi_server_config {
    long long hbm_budget_bytes;  /* device memory the live runs may hold */
    int max_live_runs;           /* slots */
    int steps_per_round;         /* steps per round (latency granularity) */
} gi_server_config;

typedef struct gi_server_request_info {
    int state;                   /* GI_REQ_* */
    int n;
    int steps_done;
    int nsteps;
    double t_submit, t_admit, t_done;  /* seconds, monotonic host clock */
    long long bytes;             /* device bytes held while live */
} gi_server_request_info;

typedef struct gi_server_stats {
    int live;
    int queued;
    long long completed;
    long long rounds;
    long long bytes_in_use;
    long long pool_bodies;       /* capacity of the device state pool */
    long long interactions;      /* pair interactions computed so far */
} gi_server_stats;

typedef struct gi_server gi_server;
/* device = GI_SERVER_DRY_RUN runs the scheduling without a GPU (states are
 * left unchanged, device memory is only accounted). */
int gi_server_create(int device, const gi_server_config *cfg, const gi_pair_params *params,
                     int nparams, gi_server **out);
int gi_server_destroy(gi_server *srv);
/* Copies the host bodies; run->offset is ignored, run->params indexes the
 * server's pair table.  GI_ERR_CAPACITY if the run alone exceeds the budget. */
int gi_server_submit(gi_server *srv, const float *pos_host, const float *vel_host,
                     const gi_run *run, int nsteps, long long *id);
/* One admit / step / retire round (synchronous). */
int gi_server_round(gi_server *srv, int *nretired);
int gi_server_query(gi_server *srv, long long id, gi_server_request_info *info);
/* Copies a finished run's bodies out and forgets the request. */
int gi_server_fetch(gi_server *srv, long long id, float *pos_host, float *vel_host);
int gi_server_get_stats(gi_server *srv, gi_server_stats *out);

/* ------------------------------------------------------------------------ */
/* Parameter helpers (host only)                                            */
/* ------------------------------------------------------------------------ */

/* The pair table the reference's loadKernalConstantStructures builds from
 * element data in code units (impactAddTime.cu:128-170,
 * generateTargetImpactor.cu:406-451): K = KFe/KSi, KR = fractions,
 * SD = shell depths as fractions of the diameter. */
int gi_params_from_material(double G, double diameter, double mass_fe,
                            double mass_si, double k_fe, double k_si,
                            double kr_fe, double kr_si, double sd_fe,
                            double sd_si, gi_pair_params *out);

/* General table from a reference collision struct (Si-Si gravity = 1). */
int gi_params_from_collision_consts(const gi_force_collision_consts *c,
                                    gi_pair_params *out);

/* ------------------------------------------------------------------------ */
/* Seeded initial conditions (host only; same bodies on every host for a    */
/* given seed).  They replace the wall-clock-seeded rand() of the           */
/* reference's body builder (generateTargetImpactorBasicFunctions.h:255).   */
/* ------------------------------------------------------------------------ */

/* n bodies uniform in a ball of the given radius; those within
 * fe_radius_fraction * radius of the centre are Fe and are placed first.
 * pos.w = tag_fe / tag_si, vel = 0, vel.w = mass.  *nfe_out = Fe count. */
int gi_ic_uniform_ball(unsigned long long seed, int n, double radius,
                       double fe_radius_fraction, float mass_fe, float mass_si,
                       float tag_fe, float tag_si, float *pos, float *vel,
                       int *nfe_out);

/* n bodies on a cubic lattice (spacing, +-jitter per axis) with Gaussian-like
 * velocities of scale vel_sigma; the first nfe are Fe.  A contact-rich test
 * configuration that exercises every band of the pair law. */
int gi_ic_lattice(unsigned long long seed, int n, double spacing, double jitter,
                  double vel_sigma, int nfe, float mass_fe, float mass_si,
                  float *pos, float *vel);

#ifdef __cplusplus
}
#endif
#endif /* GI_API_H */
