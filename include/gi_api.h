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

/* Far-field evaluation and per-body force accumulation. */
#define GI_ACCUM_PAIRED 0  /* each unordered pair once, applied to both bodies;
                              FP32 within a work item (at most 1,024 j per
                              i-body), exact 64-bit fixed point across items
                              (the default)                                  */
#define GI_ACCUM_FP32 1    /* every ordered pair; FP32 per 128-body j-tile,
                              plain FP32 across tiles                        */
#define GI_ACCUM_FP64 2    /* every ordered pair; FP32 per j-tile, FP64
                              across tiles                                   */
#define GI_ACCUM_KAHAN 3   /* every ordered pair; FP32 per j-tile,
                              Kahan-compensated across tiles                 */

typedef struct gi_options {
    int sep_test;          /* GI_SEP_*, default GI_SEP_REF_INT */
    int accum;             /* GI_ACCUM_*, 0 = GI_ACCUM_PAIRED */
    int dense_min;         /* contact pass: cells of at least this many bodies,
                              or of a quarter of it next to such a cell, take
                              the shared-memory tiled path; 0 = 256.
                              Results do not depend on it. */
    int cluster_tries;     /* gi_find_earth_moon: attempts one union-find
                              link may make (each failed attempt moves to a
                              strictly smaller root) before the call gives
                              up with GI_ERR_TIMEOUT; 0 = 2^22. */
} gi_options;

/* Work decomposition of one run (chosen per N bucket by the autotuner or
 * set explicitly).  For the one-sided modes: i_per_thread in {1, 2, 4, 8};
 * jchunk = 128 * 2^k bodies per big j-chunk (the last chunks shrink by
 * halves to 128 bodies), or 0 = the whole run in one chunk.  For
 * GI_ACCUM_PAIRED, i-blocks are 1024 bodies (8 per thread) and a work item
 * spans jchunk bodies of j, taken to 64 .. 1024 (0 = 1024); i_per_thread
 * is not used.  The result for a run depends only on these numbers and n,
 * never on what else is in the batch. */
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
 * (the reference needs n % 256 == 0).  Reference separation test, the
 * default (paired) accumulation.  Uses library-owned scratch on the current
 * device. */
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
 * All scratch lives in one static device array of 8 MiB that every GPU
 * loading the library holds until exit, so a call takes at most
 * GI_NOALLOC_MAX_BODIES bodies (larger n returns GI_ERR_BAD_SIZE).  The
 * first call on a device looks the array up (cudaGetSymbolAddress); make it
 * before any stream capture.  Calls share the array: calls that overlap on
 * the GPU (e.g. on two streams) race, so serialise them.  Forces are
 * bit-identical to gi_forces_collision's (same kernels, same default
 * decomposition). */
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
 * force pass on the caller's own bodies for every decomposition of the
 * context's accumulation mode (GI_ACCUM_PAIRED: 2^-2 .. 2^2 times the
 * default j-chunks per work item; the one-sided modes: i_per_thread in
 * {1, 2, 4} and five big-chunk sizes) and stores the fastest in the context
 * (synchronous; allocates a temporary force array).  Later calls decompose
 * runs of those buckets with the tuned values; results depend only on n and
 * this table. */
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
 * (Earth), 3 = label 2 (Moon)  (impactBasicFunctions.h:219-652), 4 = label 3
 * (the disk of gi_find_disk).
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

/* End-to-end call with HOST buffers: copies the runs' bodies of pos/vel
 * (pinned or pageable) to the device, runs nsteps fused steps, copies them
 * back, synchronises; host bodies outside the runs are neither read nor
 * changed.  What a driver does between two records
 * (impactAddTime.cu:396-431). */
int gi_run_host(gi_ctx *ctx, float *pos_host, float *vel_host, int ntotal,
                const gi_run *runs, int nruns, const gi_pair_params *params,
                int nparams, int nsteps, void *stream);

/* Measured FP32 FFMA throughput of the device in TFLOP/s (synchronous, a
 * ~50 ms microbenchmark): the denominator of the force kernel's roofline. */
int gi_measure_ffma_peak(int device, double *tflops);

/* Test hook (no counterpart in the reference): overwrites the work-queue
 * counters and split tickets of the context's scratch for `stream` with a
 * memset byte pattern (value = 0xbbbbbbbb for byte bb), as a launch that was
 * cut short would leave them; synchronous.  The next force call must still
 * be correct, because every launch clears them first. */
int gi_debug_fill_counters(gi_ctx *ctx, void *stream, unsigned int value);

/* Test hook: the paired far field's decomposition of one run of n bodies
 * with 2^pcl j-chunks per work item (pcl < 0: this context's choice, or the
 * default one when ctx is NULL); host arithmetic only, no device work.
 * out[6] = {pcl, j-chunks, i-blocks, work items, stride of the item
 * permutation, items of i-block 0}. */
int gi_debug_pair_plan(gi_ctx *ctx, int n, int pcl, long long out[6]);

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

/* Stepping policy of a round. */
#define GI_SERVE_SHARE 0     /* every live run advances each round            */
#define GI_SERVE_SHORTEST 1  /* live runs in order of least remaining work
                                (steps left x N^2) until the per-step pair
                                count reaches fill_interactions; the others
                                wait (shortest remaining work first)          */

typedef struct gi_server_config {
    long long hbm_budget_bytes;  /* device memory the live runs may hold */
    int max_live_runs;           /* slots */
    int steps_per_round;         /* steps per round (latency granularity) */
    int policy;                  /* GI_SERVE_*                             */
    long long fill_interactions; /* GI_SERVE_SHORTEST: pair interactions per
                                    step that fill the GPU; 0 = 2e9        */
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
    long long cancelled;         /* requests withdrawn by gi_server_cancel */
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
/* Withdraws a request in any state, between rounds: a queued request leaves
 * the queue; a live run gives back its slot, its device range and its share
 * of the budget at once (the other live runs are not touched); a finished
 * result is discarded.  The id is forgotten.  GI_ERR_INVALID_ARG for an
 * unknown id. */
int gi_server_cancel(gi_server *srv, long long id);

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

/* ------------------------------------------------------------------------ */
/* Setup, parameter and body files (host only)                              */
/*                                                                          */
/* Text files are read the way the reference reads them: for each value in */
/* a fixed order, skip past the next '=' and read one number; key names are */
/* not checked.  Float fields are parsed as float, double fields as double. */
/* Returns GI_ERR_IO when the file cannot be opened, GI_ERR_FORMAT when a   */
/* value is missing or not a number.                                        */
/* ------------------------------------------------------------------------ */

/* setupGeneratingTargetImpactor
 * (Code/GenerateTargetImpactorCode/generateTargetImpactor.cu:169-248). */
typedef struct gi_setup_generating {
    float spin1[4], spin2[4];          /* spin axis xyz, revolutions per hour */
    double frac_earth_mass1, frac_earth_mass2;
    double frac_fe1, frac_si1, frac_fe2, frac_si2;
    float damp1, damp2;                /* damping rates of body 1 and 2      */
    int n;                             /* TotalNumberOfElements              */
    double damp_time, damp_rest_time, spin_rest_time;  /* hours             */
    double dt;                         /* code time units                    */
    double density_fe, density_si;     /* kg km^-3                           */
    double k_fe, k_si;                 /* kg km^-1 s^-2                      */
    double kr_fe, kr_si, sd_fe, sd_si;
    int draw_rate;
} gi_setup_generating;

/* setupImpactInitialization (Code/ImpactCode/impactInitialization.cu:183-217):
 * body offsets in km and velocities in km/s (float, as the reference). */
typedef struct gi_setup_impact_init {
    float pos1[3], pos2[3], vel1[3], vel2[3];
} gi_setup_impact_init;

/* setupImpactAddTime (Code/ImpactCode/impactAddTime.cu:40-75). */
typedef struct gi_setup_add_time {
    double additional_time_days;
    double dt;
    int draw_rate, record_rate, recenter_rate;
} gi_setup_add_time;

/* targetImpactorParameters, the file that carries the code units from the
 * body builder to the impact drivers
 * (generateTargetImpactorBasicFunctions.h:688-711 writes it,
 * impactBasicFunctions.h:31-107 reads it). */
typedef struct gi_body_params {
    double unit_time, unit_length, unit_mass;  /* s, km, kg                   */
    double mass_fe, mass_si, diameter;         /* code units                  */
    double k_fe, k_si, kr_fe, kr_si, sd_fe, sd_si;
    int n, nfe1, nsi1, nfe2, nsi2;
} gi_body_params;

/* What the body builder derives from its setup (setTargetImpactorParameters,
 * generateTargetImpactor.cu:289-403). */
typedef struct gi_generation_plan {
    gi_body_params body;
    double mass_body1, mass_body2;               /* code units (MassOfBody1/2) */
    double damp_time, damp_rest_time, spin_rest_time;  /* code time units     */
    float spin1_w, spin2_w;                      /* revolutions per time unit */
    double radius_of_earth;                      /* code length units          */
} gi_generation_plan;

int gi_read_setup_generating(const char *path, gi_setup_generating *out);
int gi_read_setup_impact_init(const char *path, gi_setup_impact_init *out);
int gi_read_setup_add_time(const char *path, gi_setup_add_time *out);
int gi_read_body_params(const char *path, gi_body_params *out);
/* Same lines and "%f" / "%d" formats as the reference writer. */
int gi_write_body_params(const char *path, const gi_body_params *p);
/* viewCenteringInfo: initial centre of mass xyz, initial linear velocity xyz
 * (impactInitialization.cu:515-532, impactBasicFunctions.h:1074-1086). */
int gi_read_view_centering(const char *path, float out[6]);
int gi_write_view_centering(const char *path, const float v[6]);

/* Units, body counts and element masses from a setup (integer truncation of
 * the counts as in the reference).  GI_ERR_PARAMS when a body's Fe and Si
 * fractions do not add to 1 or there is no mass. */
int gi_derive_units(const gi_setup_generating *setup, gi_generation_plan *out);

/* The kernel constant structs the reference drivers load from the
 * parameters: collision (impactAddTime.cu:106-166) and separate
 * (generateTargetImpactor.cu:406-451), with the reference's float
 * conversions.  dt in code time units. */
int gi_collision_consts_from_body_params(const gi_body_params *b, double dt,
                                         gi_force_collision_consts *fc,
                                         gi_move_collision_consts *mc);
int gi_separate_consts_from_body_params(const gi_body_params *b, double dt,
                                        gi_force_separate_consts *fc,
                                        gi_move_separate_consts *mc);
/* Pair table of a reference separate struct (Si-Si gravity = 1). */
int gi_params_from_separate_consts(const gi_force_separate_consts *c,
                                   gi_pair_params *out);

/* targetImpactorInitialPosVel: int n, n float4 positions, n float4
 * velocities (generateTargetImpactorBasicFunctions.h:713-722).
 * gi_read_body_file with pos or vel NULL only returns the count in *n. */
int gi_write_body_file(const char *path, const float *pos, const float *vel, int n);
int gi_read_body_file(const char *path, float *pos, float *vel, int capacity, int *n);

/* impactPosVel: a sequence of frames, each float time, n float4 positions,
 * n float4 velocities (impactInitialization.cu:373-378, impactAddTime.cu:424-428).
 * gi_frames_read with frame = -1 reads the last frame, the point a resumed
 * run starts from (impactAddTime.cu:207-241).  GI_ERR_FORMAT when the file
 * size is not a whole number of frames. */
int gi_frames_append(const char *path, float time, const float *pos, const float *vel, int n);
int gi_frames_count(const char *path, int n, long long *nframes);
int gi_frames_read(const char *path, int n, long long frame, float *time, float *pos,
                   float *vel);

/* ------------------------------------------------------------------------ */
/* Body builder and impact set-up steps (host only)                         */
/* ------------------------------------------------------------------------ */

/* Raw target and impactor, order [Fe1, Si1, Fe2, Si2]
 * (createRawTargetImpactor, generateTargetImpactorBasicFunctions.h:239-405):
 * per body an Fe core of radius r1 and an Si shell from r1 + D to r2 + D,
 * r1 / r2 the radii of 2x the volume of NFe / NFe + NSi spheres at 68 %
 * packing; each element is a cube-normalised direction at a uniform radius,
 * redrawn while it is closer than D to an earlier element of its own
 * material group.  A seeded generator replaces the wall-clock-seeded rand().
 * pos.w = 0, 1, 2, 3 (Fe1, Si1, Fe2, Si2); vel = 0, vel.w = element mass.
 * *redraws (may be NULL) = the number of rejected draws. */
int gi_raw_bodies(unsigned long long seed, const gi_body_params *b, float *pos, float *vel,
                  long long *redraws);

/* Adds the spin of one body about its centre of mass (spinBody,
 * generateTargetImpactorBasicFunctions.h:407-470): body = 1 or 2, axis the
 * spin axis (normalised here; GI_ERR_PARAMS if it is zero), w the rate in
 * revolutions per code time unit. */
int gi_spin_body(float *pos, float *vel, const gi_generation_plan *plan, int body,
                 const float axis[3], float w);

/* Moves each body's centre of mass to the origin and removes its mean
 * velocity (zeroOutTargetImpactorDrift,
 * generateTargetImpactorBasicFunctions.h:472-506).  Like the reference, the
 * sums are divided by the body mass from the setup (MassOfBody1/2). */
int gi_zero_drift(float *pos, float *vel, const gi_generation_plan *plan);

/* targetImpactorStats (recordTargetImpactorStats,
 * generateTargetImpactorBasicFunctions.h:590-686). */
int gi_write_target_impactor_stats(const char *path, const gi_generation_plan *plan,
                                   const gi_setup_generating *setup, double dt,
                                   const float *pos, const float *vel);

/* Impact initial conditions (setupInitialConditions,
 * impactInitialization.cu:260-391): shift body 1 and body 2 by their setup
 * offset and velocity (converted to code units in float as the reference
 * does), then reorder [Fe1, Si1, Fe2, Si2] -> [Fe1, Fe2, Si1, Si2], so that
 * index < NFe1 + NFe2 is Fe. */
int gi_impact_initial_conditions(const gi_body_params *b, const gi_setup_impact_init *s,
                                 const float *pos_in, const float *vel_in, float *pos_out,
                                 float *vel_out);

/* Whole-system mass, centre of mass, linear velocity and angular momentum in
 * double, summed in index order as the reference's recordInitialImpactStat
 * (impactInitialization.cu:393-474): out = [mass, com xyz, vel xyz, L xyz]. */
int gi_system_stats_host(const float *pos, const float *vel, int n, int nfe, double mass_fe,
                         double mass_si, double out[10]);

/* initialStatsFile (impactInitialization.cu:476-513). stats as above. */
int gi_write_initial_stats(const char *path, const gi_body_params *b, const double stats[10]);

/* ------------------------------------------------------------------------ */
/* Earth / Moon identification and the final statistics                    */
/* ------------------------------------------------------------------------ */

/* Result of gi_find_earth_moon.  Groups are the connected sets of bodies
 * whose pairwise distance sqrtf(dx*dx + dy*dy + dz*dz) (FP32) is below
 * touch; a group is named by its smallest body index, as the reference's
 * group numbers are (findEarthAndMoon, impactBasicFunctions.h:109-217).
 * The Earth is the largest group (the smallest name on a tie), the Moon the
 * largest of the others (-1 / 0 when there is no other group).  Counts by
 * origin are [Fe body 1, Fe body 2, Si body 1, Si body 2] of the
 * [Fe1, Fe2, Si1, Si2] order (impactBasicFunctions.h:921-935). */
typedef struct gi_earth_moon {
    int earth_label, moon_label;
    int n_earth, n_moon;
    int n_groups;
    int earth_counts[4];
    int moon_counts[4];
} gi_earth_moon;

/* Groups on the GPU (hashed cell grid of cell size > touch, lock-free
 * union-find); synchronous.  pos: device, n float4.  bounds = NFe1,
 * NFe1 + NFe2, NFe1 + NFe2 + NSi1 for the origin counts.  group (device,
 * n ints, may be NULL) receives each body's group name; scope (device, n
 * bytes, may be NULL) receives 1 for Earth, 2 for Moon, 0 otherwise -- the
 * label array gi_diag_fp64 takes.  touch is 1.5 D in the reference. */
int gi_find_earth_moon(gi_ctx *ctx, const float *pos, int n, float touch, const int bounds[3],
                       int *group, unsigned char *scope, gi_earth_moon *out, void *stream);

/* The disk: bodies in neither the Earth nor the Moon that are bound to the
 * Earth -- specific orbital energy v^2/2 - G M_E / r < 0 relative to the
 * Earth's centre of mass and velocity -- and whose equivalent circular orbit
 * r_eq = h^2 / (G M_E) (h = |r x v|) lies outside the Earth's radius R_E, the
 * largest distance of an Earth element from the Earth's centre of mass plus
 * D/2.  The reference defines no disk; this is the usual definition of
 * giant-impact analyses.  Needs the scope array of gi_find_earth_moon; marks
 * disk bodies 3 in it (gi_diag_fp64 scope 4).  G is read from the pair
 * table (GMassSiSi / MassSi^2).  Synchronous; FP64. */
typedef struct gi_disk_info {
    int n_disk;            /* bound, r_eq > R_E                             */
    int n_bound_inside;    /* bound, r_eq <= R_E: falls back onto the Earth */
    int n_unbound;         /* escaping                                      */
    double earth_mass, earth_radius;
} gi_disk_info;

int gi_find_disk(gi_ctx *ctx, const float *pos, const float *vel, const gi_run *run,
                 const gi_pair_params *params, unsigned char *scope, gi_disk_info *out,
                 void *stream);

/* runStatsFile (recordFinalImpactStat, impactBasicFunctions.h:883-1072):
 * scope_stats[s] = gi_diag_fp64's out[0..9] for scope s = 0 (all),
 * 1 (Earth + Moon), 2 (Earth), 3 (Moon); time in code units. */
int gi_write_run_stats(const char *path, const gi_body_params *b, double time,
                       const gi_earth_moon *em, const double scope_stats[4][15]);

/* ------------------------------------------------------------------------ */
/* Headless pictures (the reference's GL point drawing, without GL)         */
/* ------------------------------------------------------------------------ */

/* Camera of gluLookAt(eye, center, up) + glFrustum(-half, half, -half,
 * half, near, far) (impactAddTime.cu:535-538; the reference uses eye =
 * (0, 0, 10 R_Earth), center 0, up (0, 1, 0), half 0.2, near 0.2, far 1200,
 * 1000 x 1000 pixels, 2-pixel points). */
typedef struct gi_view {
    float eye[3], center[3], up[3];
    float frustum_half, near_plane, far_plane;
    int width, height, point_size;
} gi_view;

/* The view's orthonormal eye basis as the splat uses it (FP32):
 * out = [s xyz, u xyz, f xyz, eye xyz]. */
int gi_view_basis(const gi_view *view, float out[12]);

/* Splat n elements (device float4 positions) into rgb (HOST, width x height
 * x 3 bytes, top row first): each element a point_size square coloured by
 * origin and material (Fe body 1 yellow, Fe body 2 red, Si body 1 and 2
 * browns, commonSetup.h:125-128; classes by index: < bounds[0], < bounds[1],
 * < bounds[2], rest), nearest element wins, black background.
 * Replaces drawPictureNormal's GL_POINTS (impactBasicFunctions.h:666-697).
 * Synchronous. */
int gi_splat(gi_ctx *ctx, const float *pos, int n, const int bounds[3], const gi_view *view,
             unsigned char *rgb, void *stream);

/* The analysis picture (drawAnalysisPicture, impactBasicFunctions.h:736-781,
 * its points): only the elements of scope 1 (Earth, blue) and 2 (Moon,
 * white) of the device byte array `scope`, as gi_find_earth_moon writes it,
 * splatted like gi_splat.  The reference's centre-of-mass markers and
 * angular-momentum lines are not drawn. */
int gi_splat_scope(gi_ctx *ctx, const float *pos, int n, const unsigned char *scope,
                   const gi_view *view, unsigned char *rgb, void *stream);

/* Binary PPM (P6) of an rgb image. */
int gi_write_ppm(const char *path, const unsigned char *rgb, int width, int height);

/* The viewer's playback without a window (impactViewer.cu): renders every
 * `every`-th frame of an impactPosVel file to <out_prefix><frame>.ppm.
 * *written (may be NULL) = images written. */
int gi_render_frames(int device, const char *info_dir, const char *frames_path,
                     const gi_view *view, int every, const char *out_prefix, long long *written);

/* ------------------------------------------------------------------------ */
/* Headless drivers (the reference programs without the viewer)            */
/* ------------------------------------------------------------------------ */

typedef struct gi_generate_report {
    long long steps;          /* steps taken: damped, damped rest, spin rest  */
    long long damped_steps, rest_steps, spin_steps;
    long long redraws;        /* rejected draws of the raw-body builder       */
    double seconds;           /* wall time of the step loop                   */
} gi_generate_report;

/* generateTargetImpactor without the window (generateTargetImpactor.cu:666-775):
 * reads setup_path, builds the raw bodies (seeded), runs the damped, damped
 * rest and spin rest phases with the separate-body force (the two bodies do
 * not feel each other), spinning both bodies when the spin rest starts,
 * zeroes each body's drift and writes targetImpactorStats,
 * targetImpactorParameters and targetImpactorInitialPosVel into info_dir. */
int gi_generate_target_impactor(int device, const char *setup_path, const char *info_dir,
                                unsigned long long seed, gi_generate_report *report);

/* impactInitialization (impactInitialization.cu:535-542), host only: reads
 * info_dir/targetImpactorParameters, info_dir/targetImpactorInitialPosVel and
 * setup_path, and writes impactPosVel (frame 0), initialStatsFile and
 * viewCenteringInfo into impact_info_dir. */
int gi_impact_initialize(const char *info_dir, const char *setup_path,
                         const char *impact_info_dir);

typedef struct gi_add_time_report {
    long long steps, frames_written, recenters;
    double start_time, end_time;   /* code units                             */
    double seconds;                /* wall time of the step loop             */
    gi_earth_moon earth_moon;      /* groups of the final state              */
    gi_disk_info disk;             /* disk of the final state                */
    double disk_stats[15];         /* gi_diag_fp64 of the disk (scope 4)     */
} gi_add_time_report;

/* impactAddTime without the window (impactAddTime.cu:396-579): resumes from
 * the last frame of impact_dir/ImpactInformation/impactPosVel, steps with
 * the collision force until AdditionalTime has passed, appends a frame
 * every RecordRate steps, moves the system's centre of mass and velocity
 * back to the viewCenteringInfo values every RecenterRate steps (sums in
 * FP64 on the GPU), and at the end writes impact_dir/runStatsFile and
 * rewrites viewCenteringInfo. */
int gi_impact_add_time(int device, const char *info_dir, const char *setup_path,
                       const char *impact_dir, gi_add_time_report *report);

#ifdef __cplusplus
}
#endif
#endif /* GI_API_H */
